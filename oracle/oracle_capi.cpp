// Test infrastructure: C entry points of the CPU oracle (liboracle.so).
//
// Batch drivers mirror the reference's OpenMP batch entry points
// rneaInParallel / abaInParallel (algorithm/parallel/rnea.hpp:39-84,
// algorithm/parallel/aba.hpp:40-84): `#pragma omp parallel for
// schedule(static)` over instances, one thread-private Data per thread.
// Batch arrays are instance-contiguous (the reference's column-major
// nq x batch / nv x batch matrices): instance b of q starts at q + b*nq.
// Matrix outputs are nv x nv row-major per instance.
// Precision argument: 0 = double, 1 = long double (inputs and outputs stay double).
#include <omp.h>

#include <cstdio>
#include <cstring>
#include <exception>
#include <memory>
#include <string>

#include "oracle.hpp"
#include "flop_scalar.hpp"

namespace orc {
thread_local long long FlopCounter::ops = 0;
thread_local long long FlopCounter::sincos = 0;
}  // namespace orc

using orc::Model;

namespace {
thread_local std::string g_err;

template <class T>
struct Buf {  // converts one instance's double inputs to T
  std::vector<T> x;
  void load(const double* p, int n) {
    x.resize(n);
    for (int k = 0; k < n; ++k) x[k] = T(p[k]);
  }
};
template <class T> inline void store(const std::vector<T>& src, double* dst, size_t n) {
  for (size_t k = 0; k < n; ++k) dst[k] = (double)src[k];
}

enum Func { F_RNEA = 0, F_ABA_LOCAL, F_ABA_WORLD, F_CRBA_LOCAL, F_CRBA_WORLD, F_CHOL, F_RNEA_D, F_ABA_D, F_INTEGRATE,
            F_FK, F_JAC };

template <class T> void store_placements(const orc::Data<T>& d, int nj, double* o) {  // joint 0: identity
  for (int i = 0; i < nj; ++i)
    for (int k = 0; k < 12; ++k)
      o[12 * i + k] = i == 0 ? ((k == 0 || k == 4 || k == 8) ? 1.0 : 0.0)
                             : (double)(k < 9 ? d.oMi[i].R[k] : d.oMi[i].t[k - 9]);
}
template <class T> void store_motions(const std::vector<orc::Vec6<T>>& x, int nj, double* o) {
  for (int i = 0; i < nj; ++i)
    for (int k = 0; k < 6; ++k) o[6 * i + k] = (double)x[i].v[k];
}

template <class T>
void run_one(const Model& m, orc::Data<T>& d, int func, const double* q, const double* v, const double* x,
             double* o1, double* o2, double* o3, double* o4, const double* fe = nullptr) {
  Buf<T> bq, bv, bx, bf;
  const int nq = m.nq, nv = m.nv;
  const size_t nn = (size_t)nv * nv;
  bq.load(q, nq);
  if (v) bv.load(v, nv);
  if (x) bx.load(x, nv);
  if (fe) bf.load(fe, 6 * m.njoints);
  const T* fext = fe ? bf.x.data() : nullptr;  // external forces (njoints x 6, joint frames)
  switch (func) {
    case F_RNEA:
      orc::rnea(m, d, bq.x.data(), bv.x.data(), bx.x.data(), fext);
      store(d.tau, o1, nv);
      break;
    case F_ABA_LOCAL:
    case F_ABA_WORLD:
      orc::aba(m, d, bq.x.data(), bv.x.data(), bx.x.data(), func == F_ABA_WORLD ? orc::WORLD : orc::LOCAL, fext);
      store(d.ddq, o1, nv);
      break;
    case F_CRBA_LOCAL:
    case F_CRBA_WORLD:
      std::fill(d.M.begin(), d.M.end(), T(0));
      orc::crba(m, d, bq.x.data(), func == F_CRBA_WORLD ? orc::WORLD : orc::LOCAL);
      store(d.M, o1, nn);
      break;
    case F_CHOL: {  // q holds an nv x nv row-major M (upper triangle read)
      Buf<T> bm;
      bm.load(q, (int)nn);
      d.M = bm.x;
      std::fill(d.U.begin(), d.U.end(), T(0));
      for (int k = 0; k < nv; ++k) d.U[(size_t)k * nv + k] = T(1);
      orc::cholesky_decompose(m, d);
      store(d.U, o1, nn);
      store(d.D, o2, nv);
      break;
    }
    case F_RNEA_D:
      std::fill(d.M.begin(), d.M.end(), T(0));
      std::fill(d.dtau_dq.begin(), d.dtau_dq.end(), T(0));
      std::fill(d.dtau_dv.begin(), d.dtau_dv.end(), T(0));
      orc::rnea_derivatives(m, d, bq.x.data(), bv.x.data(), bx.x.data(), fext);
      if (o1) store(d.tau, o1, nv);
      if (o2) store(d.dtau_dq, o2, nn);
      if (o3) store(d.dtau_dv, o3, nn);
      if (o4) store(d.M, o4, nn);
      break;
    case F_ABA_D:
      std::fill(d.dtau_dq.begin(), d.dtau_dq.end(), T(0));
      std::fill(d.dtau_dv.begin(), d.dtau_dv.end(), T(0));
      orc::aba_derivatives(m, d, bq.x.data(), bv.x.data(), bx.x.data(), fext);
      if (o1) store(d.ddq, o1, nv);
      if (o2) store(d.ddq_dq, o2, nn);
      if (o3) store(d.ddq_dv, o3, nn);
      if (o4) store(d.Minv, o4, nn);
      break;
    case F_FK:
      orc::forward_kinematics(m, d, bq.x.data(), v ? bv.x.data() : nullptr, (v && x) ? bx.x.data() : nullptr);
      store_placements(d, m.njoints, o1);
      if (o2) store_motions(d.v, m.njoints, o2);
      if (o3) store_motions(d.a, m.njoints, o3);
      break;
    case F_JAC:
      orc::joint_jacobians(m, d, bq.x.data());
      store(d.J, o1, (size_t)6 * nv);
      break;
    case F_INTEGRATE: {
      std::vector<T> out(nq);
      orc::integrate(m, bq.x.data(), bv.x.data(), out.data());
      store(out, o1, nq);
      break;
    }
    default:
      throw std::invalid_argument("unknown function");
  }
}

int in_stride(int func, const Model& m, int which) {  // per-instance input lengths
  if (which == 0) return func == F_CHOL ? m.nv * m.nv : m.nq;
  return m.nv;
}
int out_stride(int func, const Model& m, int which) {
  const int nn = m.nv * m.nv;
  switch (func) {
    case F_CRBA_LOCAL: case F_CRBA_WORLD: return nn;
    case F_CHOL: return which == 0 ? nn : m.nv;
    case F_RNEA_D: case F_ABA_D: return which == 0 ? m.nv : nn;
    case F_INTEGRATE: return m.nq;
    case F_FK: return which == 0 ? 12 * m.njoints : 6 * m.njoints;
    case F_JAC: return 6 * m.nv;
    default: return m.nv;
  }
}

template <class T>
int run_batch(const Model& m, int func, long B, const double* q, const double* v, const double* x, double* o1,
              double* o2, double* o3, double* o4, int nthreads, const double* fe) {
  if (nthreads <= 0) nthreads = omp_get_max_threads();
  omp_set_dynamic(0);  // set_default_omp_options (algorithm/parallel/omp.hpp:12-16)
  omp_set_num_threads(nthreads);
  const int sq = in_stride(func, m, 0), sv = in_stride(func, m, 1);
  const int s1 = out_stride(func, m, 0), s2 = out_stride(func, m, 1), s3 = out_stride(func, m, 2),
            s4 = out_stride(func, m, 3);
  std::vector<std::unique_ptr<orc::Data<T>>> datas(nthreads);  // the ModelPool's per-thread Data
  for (int t = 0; t < nthreads; ++t) datas[t].reset(new orc::Data<T>(m));
  bool failed = false;
  std::string msg;
#pragma omp parallel for schedule(static)
  for (long b = 0; b < B; ++b) {
    try {
      run_one<T>(m, *datas[omp_get_thread_num()], func, q + (size_t)b * sq, v ? v + (size_t)b * sv : nullptr,
                 x ? x + (size_t)b * sv : nullptr, o1 ? o1 + (size_t)b * s1 : nullptr,
                 o2 ? o2 + (size_t)b * s2 : nullptr, o3 ? o3 + (size_t)b * s3 : nullptr,
                 o4 ? o4 + (size_t)b * s4 : nullptr, fe ? fe + (size_t)b * 6 * m.njoints : nullptr);
    } catch (const std::exception& e) {
#pragma omp critical
      {
        failed = true;
        msg = e.what();
      }
    }
  }
  if (failed) {
    g_err = msg;
    return -1;
  }
  return 0;
}

int dispatch(void* h, int prec, int func, long B, const double* q, const double* v, const double* x, double* o1,
             double* o2, double* o3, double* o4, int nthreads, const double* fe = nullptr) {
  if (!h) { g_err = "null model"; return -1; }
  const Model& m = *static_cast<Model*>(h);
  if (prec == 0) return run_batch<double>(m, func, B, q, v, x, o1, o2, o3, o4, nthreads, fe);
  if (prec == 1) return run_batch<long double>(m, func, B, q, v, x, o1, o2, o3, o4, nthreads, fe);
  g_err = "unknown precision";
  return -1;
}
}  // namespace

extern "C" {

const char* orc_last_error() { return g_err.c_str(); }

void* orc_model_new(int njoints, const int* parents, const int* jtype, const double* placement,
                    const double* inertia, const double* armature, int nv_armature, const double* gravity,
                    const double* axis) {
  try {
    std::unique_ptr<Model> m(new Model());
    m->njoints = njoints;
    if (axis) m->axis.assign(axis, axis + 3 * njoints);
    m->parents.assign(parents, parents + njoints);
    m->jtype.assign(jtype, jtype + njoints);
    m->placement.assign(placement, placement + 12 * njoints);
    m->inertia.assign(inertia, inertia + 10 * njoints);
    if (armature) m->armature.assign(armature, armature + nv_armature);
    if (gravity) std::memcpy(m->gravity, gravity, 6 * sizeof(double));
    m->finalize();
    return m.release();
  } catch (const std::exception& e) {
    g_err = e.what();
    return nullptr;
  }
}

void orc_model_free(void* h) { delete static_cast<Model*>(h); }

int orc_model_dims(void* h, int* nq, int* nv) {
  const Model& m = *static_cast<Model*>(h);
  *nq = m.nq;
  *nv = m.nv;
  return 0;
}

// Copies the tree tables: idx_q, idx_v, nvSubtree (njoints each) and
// parents_fromRow, nvSubtree_fromRow (nv each).
int orc_model_tables(void* h, int* idx_q, int* idx_v, int* nvSubtree, int* parents_fromRow, int* nvSubtree_fromRow) {
  const Model& m = *static_cast<Model*>(h);
  for (int i = 0; i < m.njoints; ++i) { idx_q[i] = m.idx_q[i]; idx_v[i] = m.idx_v[i]; nvSubtree[i] = m.nvSubtree[i]; }
  for (int k = 0; k < m.nv; ++k) { parents_fromRow[k] = m.parents_fromRow[k]; nvSubtree_fromRow[k] = m.nvSubtree_fromRow[k]; }
  return 0;
}

int orc_rnea(void* h, int prec, long B, const double* q, const double* v, const double* a, double* tau, int nt) {
  return dispatch(h, prec, F_RNEA, B, q, v, a, tau, nullptr, nullptr, nullptr, nt);
}
int orc_aba(void* h, int prec, int conv, long B, const double* q, const double* v, const double* tau, double* ddq,
            int nt) {
  return dispatch(h, prec, conv == orc::WORLD ? F_ABA_WORLD : F_ABA_LOCAL, B, q, v, tau, ddq, nullptr, nullptr,
                  nullptr, nt);
}
int orc_crba(void* h, int prec, int conv, long B, const double* q, double* M, int nt) {
  return dispatch(h, prec, conv == orc::WORLD ? F_CRBA_WORLD : F_CRBA_LOCAL, B, q, nullptr, nullptr, M, nullptr,
                  nullptr, nullptr, nt);
}
int orc_cholesky(void* h, int prec, long B, const double* M, double* U, double* D, int nt) {
  return dispatch(h, prec, F_CHOL, B, M, nullptr, nullptr, U, D, nullptr, nullptr, nt);
}
int orc_rnea_derivatives(void* h, int prec, long B, const double* q, const double* v, const double* a, double* tau,
                         double* dtau_dq, double* dtau_dv, double* M, int nt) {
  return dispatch(h, prec, F_RNEA_D, B, q, v, a, tau, dtau_dq, dtau_dv, M, nt);
}
int orc_aba_derivatives(void* h, int prec, long B, const double* q, const double* v, const double* tau, double* ddq,
                        double* ddq_dq, double* ddq_dv, double* Minv, int nt) {
  return dispatch(h, prec, F_ABA_D, B, q, v, tau, ddq, ddq_dq, ddq_dv, Minv, nt);
}
// With external forces fext (njoints x 6 per instance, [linear; angular] in the
// joint frames): rnea / aba / computeRNEADerivatives / computeABADerivatives of
// the reference's fext overloads (algorithm/rnea.hxx:164-218, aba.hxx:296-352 and
// 543-605, rnea-derivatives.hxx:550-633, aba-derivatives.hxx:463-541).
int orc_rnea_fext(void* h, int prec, long B, const double* q, const double* v, const double* a, const double* fext,
                  double* tau, int nt) {
  return dispatch(h, prec, F_RNEA, B, q, v, a, tau, nullptr, nullptr, nullptr, nt, fext);
}
int orc_aba_fext(void* h, int prec, int conv, long B, const double* q, const double* v, const double* tau,
                 const double* fext, double* ddq, int nt) {
  return dispatch(h, prec, conv == orc::WORLD ? F_ABA_WORLD : F_ABA_LOCAL, B, q, v, tau, ddq, nullptr, nullptr,
                  nullptr, nt, fext);
}
int orc_rnea_derivatives_fext(void* h, int prec, long B, const double* q, const double* v, const double* a,
                              const double* fext, double* tau, double* dtau_dq, double* dtau_dv, double* M, int nt) {
  return dispatch(h, prec, F_RNEA_D, B, q, v, a, tau, dtau_dq, dtau_dv, M, nt, fext);
}
int orc_aba_derivatives_fext(void* h, int prec, long B, const double* q, const double* v, const double* tau,
                             const double* fext, double* ddq, double* ddq_dq, double* ddq_dv, double* Minv, int nt) {
  return dispatch(h, prec, F_ABA_D, B, q, v, tau, ddq, ddq_dq, ddq_dv, Minv, nt, fext);
}

// Contact dynamics with a given constraint Jacobian (algorithm/contact-dynamics.hxx:81-165,
// 255-327): per instance J is nc x nv row-major, gamma nc values; out = ddq (or the
// velocity after impact), lam = the multipliers.  prec 0 = double, 1 = long double.
}  // extern "C"
namespace {
template <class T>
int contact_batch(const Model& m, bool impulse, long B, int nc, const double* q, const double* v, const double* x,
                  const double* J, const double* gamma, double r_coeff, double inv_damping, double* out, double* lam,
                  int nthreads) {
  if (nthreads <= 0) nthreads = omp_get_max_threads();
  omp_set_dynamic(0);
  omp_set_num_threads(nthreads);
  std::vector<std::unique_ptr<orc::Data<T>>> datas(nthreads);
  for (int t = 0; t < nthreads; ++t) datas[t].reset(new orc::Data<T>(m));
  const int nq = m.nq, nv = m.nv;
#pragma omp parallel for schedule(static)
  for (long b = 0; b < B; ++b) {
    orc::Data<T>& d = *datas[omp_get_thread_num()];
    Buf<T> bq, bv, bx, bJ, bg;
    bq.load(q + (size_t)b * nq, nq);
    bv.load(v + (size_t)b * nv, nv);
    bJ.load(J + (size_t)b * nc * nv, nc * nv);
    std::vector<T> o(nv), l(nc);
    if (impulse) {
      orc::impulse_dynamics_contact(m, d, bq.x.data(), bv.x.data(), nc, bJ.x.data(), T(r_coeff), T(inv_damping),
                                    o.data(), l.data());
    } else {
      bx.load(x + (size_t)b * nv, nv);
      bg.load(gamma + (size_t)b * nc, nc);
      orc::forward_dynamics_contact(m, d, bq.x.data(), bv.x.data(), bx.x.data(), nc, bJ.x.data(), bg.x.data(),
                                    T(inv_damping), o.data(), l.data());
    }
    store(o, out + (size_t)b * nv, nv);
    store(l, lam + (size_t)b * nc, nc);
  }
  return 0;
}
}  // namespace
extern "C" {
int orc_forward_dynamics(void* h, int prec, long B, int nc, const double* q, const double* v, const double* tau,
                         const double* J, const double* gamma, double inv_damping, double* ddq, double* lambda_c,
                         int nt) {
  const Model& m = *static_cast<Model*>(h);
  return prec == 1 ? contact_batch<long double>(m, false, B, nc, q, v, tau, J, gamma, 0.0, inv_damping, ddq, lambda_c, nt)
                   : contact_batch<double>(m, false, B, nc, q, v, tau, J, gamma, 0.0, inv_damping, ddq, lambda_c, nt);
}
// computeKKTContactDynamicMatrixInverse (contact-dynamics.hxx:166-225), double only:
// K holds (nv + nc)^2 values per instance, row-major.
int orc_kkt_inverse(void* h, long B, int nc, const double* q, const double* J, double inv_damping, double* K) {
  const Model& m = *static_cast<Model*>(h);
  orc::Data<double> d(m);
  const size_t n = (size_t)m.nv + nc;
  for (long b = 0; b < B; ++b)
    orc::kkt_inverse_contact(m, d, q + (size_t)b * m.nq, nc, J + (size_t)b * nc * m.nv, inv_damping, K + (size_t)b * n * n);
  return 0;
}
// constraintDynamics with rigid constraint models and the proximal iterations
// (algorithm/constrained-dynamics.hxx:188-520).  Each constraint model is 46 doubles:
// type (0 = CONTACT_3D, 1 = CONTACT_6D), reference frame (1 = LOCAL, 2 = LOCAL_WORLD_ALIGNED),
// joint1, joint2, joint1_placement (R row-major, t), joint2_placement, the desired acceleration,
// Kp, Kd.  Outputs per instance: ddq (nv), lambda_c (the stacked constraint sizes), the
// iteration count and (absolute, relative) residuals.  prec 0 = double, 1 = long double.
int orc_constraint_dynamics(void* h, int prec, long B, int ncontacts, const double* desc, const double* q,
                            const double* v, const double* tau, double mu, int max_iter, double abs_acc,
                            double rel_acc, double* ddq, double* lambda_c, int* iters, double* residuals, int nt);
int orc_impulse_dynamics(void* h, int prec, long B, int nc, const double* q, const double* v_before, const double* J,
                         double r_coeff, double inv_damping, double* dq_after, double* impulse_c, int nt) {
  const Model& m = *static_cast<Model*>(h);
  return prec == 1 ? contact_batch<long double>(m, true, B, nc, q, v_before, nullptr, J, nullptr, r_coeff, inv_damping,
                                                dq_after, impulse_c, nt)
                   : contact_batch<double>(m, true, B, nc, q, v_before, nullptr, J, nullptr, r_coeff, inv_damping,
                                           dq_after, impulse_c, nt);
}

int orc_forward_kinematics(void* h, int prec, long B, const double* q, const double* v, const double* a, double* oMi,
                           double* vi, double* ai, int nt) {
  return dispatch(h, prec, F_FK, B, q, v, a, oMi, vi, ai, nullptr, nt);
}
int orc_joint_jacobians(void* h, int prec, long B, const double* q, double* J, int nt) {
  return dispatch(h, prec, F_JAC, B, q, nullptr, nullptr, J, nullptr, nullptr, nullptr, nt);
}
int orc_integrate(void* h, int prec, long B, const double* q, const double* v, double* qout, int nt) {
  return dispatch(h, prec, F_INTEGRATE, B, q, v, nullptr, qout, nullptr, nullptr, nullptr, nt);
}

// Counts the floating-point operations of one evaluation of `func` at the
// given instance (q, v, x); returns {ops, sincos pairs}.
int orc_count_flops(void* h, int func, const double* q, const double* v, const double* x, double* ops,
                    double* sincos) {
  try {
    const Model& m = *static_cast<Model*>(h);
    orc::Data<orc::FlopScalar> d(m);
    std::vector<double> o1((size_t)m.nv * m.nv + m.nq), o2((size_t)m.nv * m.nv), o3((size_t)m.nv * m.nv),
        o4((size_t)m.nv * m.nv);
    orc::FlopCounter::ops = 0;
    orc::FlopCounter::sincos = 0;
    run_one<orc::FlopScalar>(m, d, func, q, v, x, o1.data(), o2.data(), o3.data(), o4.data());
    *ops = (double)orc::FlopCounter::ops;
    *sincos = (double)orc::FlopCounter::sincos;
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

}  // extern "C"

namespace {
std::vector<orc::ConstraintModel> constraint_models(const Model& m, int n, const double* desc) {
  std::vector<orc::ConstraintModel> cms(n);
  for (int e = 0; e < n; ++e) {
    const double* d = desc + 46 * e;
    orc::ConstraintModel& c = cms[e];
    c.type = (int)d[0];
    c.frame = (int)d[1];
    c.joint1 = (int)d[2];
    c.joint2 = (int)d[3];
    std::memcpy(c.P1, d + 4, sizeof(c.P1));
    std::memcpy(c.P2, d + 16, sizeof(c.P2));
    std::memcpy(c.desired_acc, d + 28, sizeof(c.desired_acc));
    std::memcpy(c.Kp, d + 34, sizeof(c.Kp));
    std::memcpy(c.Kd, d + 40, sizeof(c.Kd));
    c.init(m);
  }
  return cms;
}
template <class T>
int constraint_batch(const Model& m, long B, const std::vector<orc::ConstraintModel>& cms, const double* q,
                     const double* v, const double* tau, double mu, int max_iter, double abs_acc, double rel_acc,
                     double* ddq, double* lam, int* iters, double* residuals, int nthreads) {
  if (nthreads <= 0) nthreads = omp_get_max_threads();
  omp_set_dynamic(0);
  omp_set_num_threads(nthreads);
  std::vector<std::unique_ptr<orc::Data<T>>> datas(nthreads);
  for (int t = 0; t < nthreads; ++t) datas[t].reset(new orc::Data<T>(m));
  int nc = 0;
  for (const auto& c : cms) nc += c.size();
  const int nq = m.nq, nv = m.nv;
#pragma omp parallel for schedule(static)
  for (long b = 0; b < B; ++b) {
    orc::Data<T>& d = *datas[omp_get_thread_num()];
    Buf<T> bq, bv, bt;
    bq.load(q + (size_t)b * nq, nq);
    bv.load(v + (size_t)b * nv, nv);
    bt.load(tau + (size_t)b * nv, nv);
    std::vector<T> o(nv), l(nc);
    const orc::ProximalResult r = orc::constraint_dynamics(m, d, bq.x.data(), bv.x.data(), bt.x.data(), cms, T(mu),
                                                           max_iter, T(abs_acc), T(rel_acc), o.data(), l.data());
    store(o, ddq + (size_t)b * nv, nv);
    store(l, lam + (size_t)b * nc, nc);
    if (iters) iters[b] = r.iter;
    if (residuals) {
      residuals[2 * b] = r.absolute_residual;
      residuals[2 * b + 1] = r.relative_residual;
    }
  }
  return 0;
}
}  // namespace
extern "C" int orc_constraint_dynamics(void* h, int prec, long B, int ncontacts, const double* desc, const double* q,
                                       const double* v, const double* tau, double mu, int max_iter, double abs_acc,
                                       double rel_acc, double* ddq, double* lambda_c, int* iters, double* residuals,
                                       int nt) {
  const Model& m = *static_cast<Model*>(h);
  try {
    const std::vector<orc::ConstraintModel> cms = constraint_models(m, ncontacts, desc);
    if (max_iter < 1 || !(mu >= 0.0)) throw std::invalid_argument("max_iter must be >= 1 and mu >= 0");
    return prec == 1 ? constraint_batch<long double>(m, B, cms, q, v, tau, mu, max_iter, abs_acc, rel_acc, ddq,
                                                     lambda_c, iters, residuals, nt)
                     : constraint_batch<double>(m, B, cms, q, v, tau, mu, max_iter, abs_acc, rel_acc, ddq, lambda_c,
                                                iters, residuals, nt);
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

// log6 and Jlog6 of one placement M (12 doubles: R row-major, t): xi (6), J (6 x 6 row-major)
extern "C" int orc_log6(const double* M, double* xi, double* J) {
  orc::SE3<double> P = orc::se3_from<double>(M);
  const orc::Vec6<double> x = orc::log6(P);
  for (int k = 0; k < 6; ++k) xi[k] = x.v[k];
  if (J) orc::jlog6(P, J);
  return 0;
}

// ContactCholeskyDecomposition(model, contact_models).compute(model, data, contact_models,// ContactCholeskyDecomposition(model, contact_models).compute(model, data, contact_models,
// contact_datas, mu) at each configuration and its accessors (contact-cholesky.hpp:168-265,
// contact-cholesky.hxx:152-304, 617-759); n = constraint dim + nv; every output may be null.
extern "C" int orc_contact_cholesky(void* h, long B, int ncontacts, const double* desc, const double* q, double mu,
                                    double* kkt, double* kkt_inv, double* osim_inv, double* osim, double* minv,
                                    double* jminv, int nt) {
  const Model& m = *static_cast<Model*>(h);
  try {
    const std::vector<orc::ConstraintModel> cms = constraint_models(m, ncontacts, desc);
    if (!(mu >= 0.0)) throw std::invalid_argument("mu must be positive.");
    int nc = 0;
    for (const auto& c : cms) nc += c.size();
    const size_t n = (size_t)nc + m.nv, nv = m.nv;
    if (nt <= 0) nt = omp_get_max_threads();
    omp_set_dynamic(0);
    omp_set_num_threads(nt);
    std::vector<std::unique_ptr<orc::Data<double>>> datas(nt);
    for (int t = 0; t < nt; ++t) datas[t].reset(new orc::Data<double>(m));
#pragma omp parallel for schedule(static)
    for (long b = 0; b < B; ++b) {
      auto at = [&](double* p, size_t k) { return p ? p + (size_t)b * k : nullptr; };
      orc::contact_cholesky(m, *datas[omp_get_thread_num()], q + (size_t)b * m.nq, cms, mu, at(kkt, n * n),
                            at(kkt_inv, n * n), at(osim_inv, (size_t)nc * nc), at(osim, (size_t)nc * nc),
                            at(minv, nv * nv), at(jminv, (size_t)nc * nv));
    }
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

namespace {
template <class T>
int constraint_derivs_batch(const Model& m, long B, const std::vector<orc::ConstraintModel>& cms, const double* q,
                            const double* v, const double* tau, double mu, int max_iter, double abs_acc,
                            double rel_acc, double* ddq, double* lam, double* ddq_dq, double* ddq_dv,
                            double* ddq_dtau, double* dl_dq, double* dl_dv, double* dl_dtau, int* iters,
                            int nthreads) {
  if (nthreads <= 0) nthreads = omp_get_max_threads();
  omp_set_dynamic(0);
  omp_set_num_threads(nthreads);
  std::vector<std::unique_ptr<orc::Data<T>>> datas(nthreads);
  for (int t = 0; t < nthreads; ++t) datas[t].reset(new orc::Data<T>(m));
  int nc = 0;
  for (const auto& c : cms) nc += c.size();
  const int nq = m.nq, nv = m.nv;
  const size_t nn = (size_t)nv * nv, cn = (size_t)nc * nv;
  std::string err;
#pragma omp parallel for schedule(static)
  for (long b = 0; b < B; ++b) {
    orc::Data<T>& d = *datas[omp_get_thread_num()];
    Buf<T> bq, bv, bt;
    bq.load(q + (size_t)b * nq, nq);
    bv.load(v + (size_t)b * nv, nv);
    bt.load(tau + (size_t)b * nv, nv);
    std::vector<T> o(nv), l(nc), a1(nn), a2(nn), a3(nn), l1(cn), l2(cn), l3(cn);
    try {
      const orc::ProximalResult r = orc::constraint_dynamics_derivatives(
          m, d, bq.x.data(), bv.x.data(), bt.x.data(), cms, T(mu), max_iter, T(abs_acc), T(rel_acc), o.data(),
          l.data(), a1.data(), a2.data(), a3.data(), l1.data(), l2.data(), l3.data());
      if (iters) iters[b] = r.iter;
    } catch (const std::exception& e) {
#pragma omp critical
      err = e.what();
      continue;
    }
    store(o, ddq + (size_t)b * nv, nv);
    store(l, lam + (size_t)b * nc, nc);
    store(a1, ddq_dq + b * nn, nn);
    store(a2, ddq_dv + b * nn, nn);
    store(a3, ddq_dtau + b * nn, nn);
    store(l1, dl_dq + b * cn, cn);
    store(l2, dl_dv + b * cn, cn);
    store(l3, dl_dtau + b * cn, cn);
  }
  if (!err.empty()) throw std::invalid_argument(err);
  return 0;
}
}  // namespace
// computeConstraintDynamicsDerivatives (algorithm/constrained-dynamics-derivatives.hxx:344-1050) for
// constraints to the world without Baumgarte gains: per instance ddq, lambda_c, ddq_dq, ddq_dv,
// ddq_dtau (nv x nv), dlambda_dq, dlambda_dv, dlambda_dtau (nc x nv), row-major, and the iterations.
extern "C" int orc_constraint_dynamics_derivatives(void* h, int prec, long B, int ncontacts, const double* desc,
                                                   const double* q, const double* v, const double* tau, double mu,
                                                   int max_iter, double abs_acc, double rel_acc, double* ddq,
                                                   double* lambda_c, double* ddq_dq, double* ddq_dv, double* ddq_dtau,
                                                   double* dl_dq, double* dl_dv, double* dl_dtau, int* iters, int nt) {
  const Model& m = *static_cast<Model*>(h);
  try {
    const std::vector<orc::ConstraintModel> cms = constraint_models(m, ncontacts, desc);
    if (max_iter < 1 || !(mu >= 0.0)) throw std::invalid_argument("max_iter must be >= 1 and mu >= 0");
    return prec == 1 ? constraint_derivs_batch<long double>(m, B, cms, q, v, tau, mu, max_iter, abs_acc, rel_acc, ddq,
                                                            lambda_c, ddq_dq, ddq_dv, ddq_dtau, dl_dq, dl_dv, dl_dtau,
                                                            iters, nt)
                     : constraint_derivs_batch<double>(m, B, cms, q, v, tau, mu, max_iter, abs_acc, rel_acc, ddq,
                                                       lambda_c, ddq_dq, ddq_dv, ddq_dtau, dl_dq, dl_dv, dl_dtau,
                                                       iters, nt);
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}
