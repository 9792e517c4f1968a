// Test infrastructure: host (CPU) build of the per-instance kernel code in
// pinocchio_gb300/csrc/gb_dyn.cuh, so that the kernel arithmetic -- including
// the mixed-precision split -- can be checked against the oracle without a
// GPU.  The product never links this file.
#define _GNU_SOURCE 1
#include <math.h>

#include <string>

#include "../../pinocchio_gb300/csrc/gb_dyn.cuh"
#include "../../pinocchio_gb300/csrc/gb_model_build.h"

namespace {
thread_local std::string g_err;
gb::In in_at(const double* p, long b, long n) { return gb::In{p + b * n, 1}; }
gb::Out out_at(double* p, long b, long n) { return gb::Out{p + b * n, 1}; }
double to_double(double x) { return x; }
double to_double(float x) { return x; }
double to_double(gb::dfloat x) { return double(x.hi) + double(x.lo); }
}  // namespace

extern "C" {
const char* hs_last_error() { return g_err.c_str(); }

void* hs_model_new(const gb_model_desc* d) {
  gb_model* M = new gb_model();
  if (gbm::build_model(M, d, &g_err) != GB_OK) {
    delete M;
    return nullptr;
  }
  return M;
}
void hs_model_free(void* h) { delete static_cast<gb_model*>(h); }

#define HS_DISPATCH(CAPV, CALL)                                            \
  switch (CAPV) {                                                          \
    case 8: { constexpr int C = 8; CALL; break; }                          \
    case 16: { constexpr int C = 16; CALL; break; }                        \
    case 32: { constexpr int C = 32; CALL; break; }                        \
    case 64: { constexpr int C = 64; CALL; break; }                        \
    default: { constexpr int C = 128; CALL; break; }                       \
  }

// fext: external forces (njoints x 6 per instance) or NULL
int hs_rnea(void* h, int mixed, long B, const double* q, const double* v, const double* a, double* tau,
            const double* fext) {
  const gb_model* M = static_cast<gb_model*>(h);
  const gb::MView m = gb::make_view(M->blob.data());
#pragma omp parallel for schedule(static)
  for (long b = 0; b < B; ++b) {
    const gb::In fe = in_at(fext, b, 6L * m.nj);
    const gb::In* fp = fext ? &fe : nullptr;
    if (mixed) { HS_DISPATCH(M->cap, (gb::rnea_one<float, C>(m, in_at(q, b, m.nq), in_at(v, b, m.nv), in_at(a, b, m.nv), out_at(tau, b, m.nv), fp))); }
    else { HS_DISPATCH(M->cap, (gb::rnea_one<double, C>(m, in_at(q, b, m.nq), in_at(v, b, m.nv), in_at(a, b, m.nv), out_at(tau, b, m.nv), fp))); }
  }
  return 0;
}
int hs_aba(void* h, int mixed, long B, const double* q, const double* v, const double* tau, double* ddq,
           const double* fext) {
  const gb_model* M = static_cast<gb_model*>(h);
  const gb::MView m = gb::make_view(M->blob.data());
#pragma omp parallel for schedule(static)
  for (long b = 0; b < B; ++b) {
    const gb::In fe = in_at(fext, b, 6L * m.nj);
    const gb::In* fp = fext ? &fe : nullptr;
    if (mixed) { HS_DISPATCH(M->cap, (gb::aba_one<float, double, C, true>(m, in_at(q, b, m.nq), in_at(v, b, m.nv), in_at(tau, b, m.nv), out_at(ddq, b, m.nv), fp))); }
    else { HS_DISPATCH(M->cap, (gb::aba_one<double, double, C, true>(m, in_at(q, b, m.nq), in_at(v, b, m.nv), in_at(tau, b, m.nv), out_at(ddq, b, m.nv), fp))); }
  }
  return 0;
}
int hs_crba(void* h, int mixed, int symmetric, long B, const double* q, double* Mo, double* U, double* D) {
  const gb_model* M = static_cast<gb_model*>(h);
  const gb::MView m = gb::make_view(M->blob.data());
  const long nn = (long)m.nv * m.nv;
#pragma omp parallel for schedule(static)
  for (long b = 0; b < B; ++b) {
    const gb::Out Uo = U ? out_at(U, b, nn) : gb::Out{nullptr, 1};
    const gb::Out Do = D ? out_at(D, b, m.nv) : gb::Out{nullptr, 1};
    if (mixed) { HS_DISPATCH(M->cap, (gb::crba_one<float, C>(m, in_at(q, b, m.nq), out_at(Mo, b, nn), symmetric != 0, U ? &Uo : nullptr, U ? &Do : nullptr, false))); }
    else { HS_DISPATCH(M->cap, (gb::crba_one<double, C>(m, in_at(q, b, m.nq), out_at(Mo, b, nn), symmetric != 0, U ? &Uo : nullptr, U ? &Do : nullptr, false))); }
  }
  return 0;
}
int hs_integrate(void* h, long B, const double* q, const double* v, double* qo) {
  const gb_model* M = static_cast<gb_model*>(h);
  const gb::MView m = gb::make_view(M->blob.data());
#pragma omp parallel for schedule(static)
  for (long b = 0; b < B; ++b) gb::integrate_one(m, in_at(q, b, m.nq), in_at(v, b, m.nv), out_at(qo, b, m.nq));
  return 0;
}
}

// ---- derivatives (host build of gb_derivs.cuh; the workspace is per instance, stride 1) ----
#include "../../pinocchio_gb300/csrc/gb_derivs.cuh"
#include <vector>

extern "C" int hs_rnea_derivs(void* h, int mixed, int symmetric, long B, const double* q, const double* v, const double* a,
                   double* dq, double* dv, double* Mo, double* tau, const double* fext) {
  const gb_model* M = static_cast<gb_model*>(h);
  const gb::MView m = gb::make_view(M->blob.data());
  const gb::DerivLayout L = gb::make_deriv_layout(m.nj, m.nv, M->nslot, false);
  const long nn = (long)m.nv * m.nv;
#pragma omp parallel
  {
    std::vector<double> wd(L.nS);
    std::vector<float> wf(L.nS);
#pragma omp for schedule(static)
    for (long b = 0; b < B; ++b) {
      const gb::Out to = out_at(tau, b, m.nv);
      const gb::In fe = in_at(fext, b, 6L * m.nj);
      const gb::In* fp = fext ? &fe : nullptr;
      if (mixed)
        gb::rnea_derivs_one<float, true>(m, L, gb::Ws<float>{wf.data(), 1}, in_at(q, b, m.nq), in_at(v, b, m.nv), in_at(a, b, m.nv),
                                   out_at(dq, b, nn), out_at(dv, b, nn), out_at(Mo, b, nn), &to, symmetric != 0, false, fp);
      else
        gb::rnea_derivs_one<double, true>(m, L, gb::Ws<double>{wd.data(), 1}, in_at(q, b, m.nq), in_at(v, b, m.nv), in_at(a, b, m.nv),
                                    out_at(dq, b, nn), out_at(dv, b, nn), out_at(Mo, b, nn), &to, symmetric != 0, false, fp);
    }
  }
  return 0;
}

// Mirrors the device: sweeps with S (column-set storage), T3 / T (column-set
// arithmetic of passes 3 / 4), K (kinematics, Minv), SS = double (Schur), P
// (dtau); then the product kernel, which writes Minv from the packed K copy
// and forms -Minv * dtau in P over the structurally non-zero rows.
template <class S, class T3, class T, class K, class P>
static void aba_derivs_host(const gb_model* M, const gb::MView& m, long b, const double* q, const double* v,
                            const double* tau, double* dq, double* dv, double* Minv, double* ddq,
                            std::vector<S>& wS, std::vector<K>& wK, std::vector<double>& wSS, const double* fext) {
  const gb::DerivLayout L = gb::make_deriv_layout(m.nj, m.nv, M->nslot, true);
  const int nv = m.nv;
  const long nn = (long)nv * nv;
  std::vector<P> wP(L.nP);
  const gb::Out dd = out_at(ddq, b, nv);
  const gb::In fe = in_at(fext, b, 6L * m.nj);
  std::vector<K> wM(nv * (nv + 1) / 2);
  gb::aba_derivs_sweeps<S, T3, T, K, double, P, true>(m, L, m.slot, gb::Ws<S>{wS.data(), 1}, gb::Ws<K>{wK.data(), 1},
                                                gb::Ws<double>{wSS.data(), 1}, gb::Ws<K>{wM.data(), 1},
                                                gb::Ws<P>{wP.data(), 1}, in_at(q, b, m.nq), in_at(v, b, nv),
                                                in_at(tau, b, nv), &dd, fext ? &fe : nullptr);
  double* Mi = Minv + b * nn;
  std::vector<P> Mp(nn);
  for (int r = 0; r < nv; ++r)
    for (int c = 0; c < nv; ++c) {
      const K x = wM[r <= c ? gb::upk(nv, r, c) : gb::upk(nv, c, r)];
      Mi[r * nv + c] = to_double(x);
      Mp[r * nv + c] = P(x);
    }
  for (int mm = 0; mm < 2; ++mm) {
    const P* X = wP.data() + (mm == 0 ? L.dtq : L.dtv);
    double* O = (mm == 0 ? dq : dv) + b * nn;
    for (int c = 0; c < nv; ++c)
      for (int r = 0; r < nv; ++r) {
        P acc = P(0);
        for (int kk = M->rel_off[c]; kk < M->rel_off[c + 1]; ++kk) {
          const int k = M->rel_list[kk];
          acc += Mp[k * nv + r] * X[k * nv + c];
        }
        O[r * nv + c] = -double(acc);
      }
  }
}

extern "C" int hs_aba_derivs(void* h, int mixed, long B, const double* q, const double* v, const double* tau, double* dq,
                  double* dv, double* Minv, double* ddq, const double* fext) {
  const gb_model* M = static_cast<gb_model*>(h);
  const gb::MView m = gb::make_view(M->blob.data());
  const gb::DerivLayout L = gb::make_deriv_layout(m.nj, m.nv, M->nslot, true);
#pragma omp parallel
  {
    std::vector<double> wd(L.nS), wdk(L.nK), wss(L.nSS);
    std::vector<float> wf(L.nS);
    std::vector<gb::dfloat> wfk(L.nK);
#pragma omp for schedule(static)
    for (long b = 0; b < B; ++b) {
      if (mixed)
        aba_derivs_host<float, float, gb::dfloat, gb::dfloat, float>(M, m, b, q, v, tau, dq, dv, Minv, ddq, wf, wfk, wss,
                                                                     fext);
      else aba_derivs_host<double, double, double, double, double>(M, m, b, q, v, tau, dq, dv, Minv, ddq, wd, wdk, wss,
                                                                   fext);
    }
  }
  return 0;
}
