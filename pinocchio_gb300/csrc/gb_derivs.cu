// Batched analytical derivatives: computeRNEADerivatives and computeABADerivatives.
//
// RNEA derivatives: one kernel, one thread per configuration.
// ABA derivatives: (1) a sweep kernel (one thread per configuration) that
// produces ddq, the symmetric Minv and dtau_dq / dtau_dv at (q, v, ddq) in the
// workspace; (2) a CTA-cooperative kernel for ddq_dq = -Minv dtau_dq and
// ddq_dv = -Minv dtau_dv (reference algorithm/aba-derivatives.hxx:451-452):
// G configurations are staged in shared memory, one warp owns one output
// matrix, its lanes own rows, and for every column c the warp loops only over
// the rows k that can be non-zero in column c of dtau (ancestors and subtree
// of c) -- the reference multiplies the dense matrices.
#include "gb_derivs.cuh"
#include "gb_internal.h"

namespace gbi {
namespace {

constexpr int kThreads = 128;

__device__ __forceinline__ gb::MView stage_model(const unsigned char* __restrict__ blob, int bytes,
                                                 unsigned char* smem) {
  const uint4* src = reinterpret_cast<const uint4*>(blob);
  uint4* dst = reinterpret_cast<uint4*>(smem);
  for (int k = threadIdx.x; k < bytes / 16; k += blockDim.x) dst[k] = src[k];
  __syncthreads();
  return gb::make_view(smem);
}
__device__ __forceinline__ gb::In in_at(const Arr& a, long b) { return gb::In{a.p + b * a.is, a.es}; }
__device__ __forceinline__ gb::Out out_at(const Arr& a, long b) {
  return gb::Out{const_cast<double*>(a.p) + b * a.is, a.es};
}

template <class S>
__global__ void __launch_bounds__(kThreads) k_rnea_derivs(const unsigned char* blob, int bytes, long B,
                                                          gb::DerivLayout L, S* ws, bool symmetric, Arr q, Arr v,
                                                          Arr a, Arr dq, Arr dv, Arr Mo, Arr tau) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_model(blob, bytes, smem);
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const gb::Ws<S> w{ws + b, B};
  const gb::Out to = out_at(tau, b);
  gb::rnea_derivs_one<S>(m, L, w, in_at(q, b), in_at(v, b), in_at(a, b), out_at(dq, b), out_at(dv, b), out_at(Mo, b),
                         tau.p ? &to : nullptr, symmetric);
}

// The ABA-derivative sweeps as three kernels (passes 1-2, pass 3, pass 4), so
// that each keeps fewer values live than one fused kernel would (register use
// bounds the number of resident warps).  The workspace carries everything
// between them.
template <class S, class SS>
__global__ void __launch_bounds__(kThreads) k_aba_derivs_pass12(const unsigned char* blob, int bytes, long B,
                                                                gb::DerivLayout L, SS* wsSS, Arr q, Arr v, Arr tau,
                                                                Arr Minv) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_model(blob, bytes, smem);
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  gb::aba_derivs_pass12<S, SS>(m, L, gb::Ws<SS>{wsSS + b, B}, in_at(q, b), in_at(v, b), in_at(tau, b),
                               out_at(Minv, b));
}

template <class S, class SS>
__global__ void __launch_bounds__(kThreads) k_aba_derivs_pass3(const unsigned char* blob, int bytes, long B,
                                                               gb::DerivLayout L, S* wsS, SS* wsSS, Arr v, Arr Minv,
                                                               Arr ddq) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_model(blob, bytes, smem);
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const gb::Out dd = out_at(ddq, b);
  gb::aba_derivs_pass3<S, SS>(m, L, m.slot, gb::Ws<S>{wsS + b, B}, gb::Ws<SS>{wsSS + b, B}, in_at(v, b),
                              out_at(Minv, b), ddq.p ? &dd : nullptr);
}

template <class S, class SS, class P>
__global__ void __launch_bounds__(kThreads) k_aba_derivs_pass4(const unsigned char* blob, int bytes, long B,
                                                               gb::DerivLayout L, S* wsS, SS* wsSS, P* wsP,
                                                               Arr Minv) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_model(blob, bytes, smem);
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  gb::aba_derivs_pass4<S, SS, P>(m, L, gb::Ws<S>{wsS + b, B}, gb::Ws<SS>{wsSS + b, B}, gb::Ws<P>{wsP + b, B},
                                 out_at(Minv, b));
}

// out_m = -Minv * X_m for the two matrices X_0 = dtau_dq, X_1 = dtau_dv of G
// consecutive configurations per iteration.  smem: Minv[G][nv*nv], then
// X[G][NM][nv*nv] (scalar S), then the column-group tables.  NM = number of the
// two products done per pass.  A warp owns one (configuration, matrix, column
// group); its lanes own rows (lane + 32*chunk); for every row k that can be
// non-zero in the group's columns it loads one Minv row segment (lane-contiguous,
// Minv symmetric) and the group's <= 8 entries of X's row k (broadcast) and does
// up to 8 FMAs per lane.  The result overwrites the group's columns of X in place.
template <class S, class W>
__global__ void k_minv_products(const unsigned char* blob, int bytes, long B, int G, int m0, int NM, Arr Minv,
                                const W* ws, long dtq, long dtv, Arr out0, Arr out1) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const gb::BlobHeader* h = reinterpret_cast<const gb::BlobHeader*>(blob);
  const int nv = h->nv, ng = h->ngroup, nrel = h->n_grp_rel;
  const int nn = nv * nv;
  S* sM = reinterpret_cast<S*>(smem_raw);
  S* sX = sM + (long)G * nn;
  int* sgrp = reinterpret_cast<int*>(sX + (long)G * NM * nn);
  int* srel = sgrp + 4 * ng;
  for (int t = threadIdx.x; t < 4 * ng; t += blockDim.x) sgrp[t] = reinterpret_cast<const int*>(blob + h->o_grp)[t];
  for (int t = threadIdx.x; t < nrel; t += blockDim.x) srel[t] = reinterpret_cast<const int*>(blob + h->o_grp_rel)[t];
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32, nwarps = blockDim.x / 32;
  for (long b0 = (long)blockIdx.x * G; b0 < B; b0 += (long)gridDim.x * G) {
    const int g_here = (int)min((long)G, B - b0);
    __syncthreads();
    // stage Minv (caller layout) and the dtau matrices (workspace, SoA over the batch)
    for (int t = threadIdx.x; t < g_here * nn; t += blockDim.x) {
      const int g = t / nn, e = t % nn;
      sM[g * nn + e] = S(Minv.p[(b0 + g) * Minv.is + (long)e * Minv.es]);
    }
    for (int mm = 0; mm < NM; ++mm) {
      const long off = (m0 + mm) == 0 ? dtq : dtv;
      for (int t = threadIdx.x; t < g_here * nn; t += blockDim.x) {
        const int g = t % g_here, e = t / g_here;
        sX[(g * NM + mm) * nn + e] = S(ws[(off + e) * B + b0 + g]);
      }
    }
    __syncthreads();
    const int ntask = g_here * NM * ng;
    for (int task = warp; task < ntask; task += nwarps) {
      const int g = task / (NM * ng), rem = task % (NM * ng), mm = rem / ng, gi = rem % ng;
      const int c0 = sgrp[4 * gi], nc = sgrp[4 * gi + 1], k0 = sgrp[4 * gi + 2], k1 = sgrp[4 * gi + 3];
      const S* Mg = sM + g * nn;
      S* X = sX + (g * NM + mm) * nn;
      S acc[4][8];
#pragma unroll
      for (int ch = 0; ch < 4; ++ch)
#pragma unroll
        for (int c = 0; c < 8; ++c) acc[ch][c] = S(0);
      for (int kk = k0; kk < k1; ++kk) {
        const int k = srel[kk];
        const S* Xk = X + k * nv + c0;
        S x[8];
#pragma unroll
        for (int c = 0; c < 8; ++c) x[c] = c < nc ? Xk[c] : S(0);
        const S* Mk = Mg + k * nv;
#pragma unroll
        for (int ch = 0; ch < 4; ++ch) {
          const int r = ch * 32 + lane;
          if (ch * 32 < nv) {
            const S mr = r < nv ? Mk[r] : S(0);
#pragma unroll
            for (int c = 0; c < 8; ++c) acc[ch][c] += mr * x[c];
          }
        }
      }
      __syncwarp();
#pragma unroll
      for (int ch = 0; ch < 4; ++ch) {
        const int r = ch * 32 + lane;
        if (r < nv)
#pragma unroll
          for (int c = 0; c < 8; ++c)
            if (c < nc) X[r * nv + c0 + c] = -acc[ch][c];
      }
      __syncwarp();
    }
    __syncthreads();
    for (int mm = 0; mm < NM; ++mm) {
      const Arr& o = (m0 + mm) == 0 ? out0 : out1;
      double* op = const_cast<double*>(o.p);
      for (int t = threadIdx.x; t < g_here * nn; t += blockDim.x) {
        const int g = t / nn, e = t % nn;
        op[(b0 + g) * o.is + (long)e * o.es] = double(sX[(g * NM + mm) * nn + e]);
      }
    }
  }
}

int blob_smem(const gb_model* M, const void* kernel, const char* name) {
  if (M->blob_bytes > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, M->blob_bytes);
    if (e != cudaSuccess) return cuda_error(e, name);
  }
  return GB_OK;
}

// workspace: stream-ordered allocation from the device's default memory pool
struct Workspace {
  void* p = nullptr;
  cudaStream_t st = nullptr;
  ~Workspace() {
    if (p) cudaFreeAsync(p, st);
  }
};
int ws_alloc(Workspace& w, size_t bytes, cudaStream_t st) {
  w.st = st;
  static bool pool_tuned = false;
  if (!pool_tuned) {  // keep freed blocks in the pool: repeated calls reuse them
    int dev = 0;
    cudaMemPool_t pool;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      unsigned long long thr = ~0ull;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    pool_tuned = true;
  }
  return cuda_error(cudaMallocAsync(&w.p, bytes, st), "workspace allocation");
}

// S: scalar of the products (smem, FMA); W: scalar of the dtau matrices in the workspace
template <class S, class W>
int launch_minv_products(const gb_model* M, long B, Arr Minv, const W* ws, const gb::DerivLayout& L, Arr o0, Arr o1,
                         cudaStream_t st) {
  const long nn = (long)M->nv * M->nv;
  const long budget = 190 * 1024;
  int NM = 2;
  long G = budget / (nn * (long)sizeof(S) * (1 + NM));
  if (G < 1) {
    NM = 1;
    G = budget / (nn * (long)sizeof(S) * (1 + NM));
  }
  if (G < 1) return set_error(GB_ERR_UNSUPPORTED, "nv too large for the Minv products");
  G = std::min<long>(G, 16);
  const int ngroup = reinterpret_cast<const gb::BlobHeader*>(M->blob.data())->ngroup;
  const int nrel = reinterpret_cast<const gb::BlobHeader*>(M->blob.data())->n_grp_rel;
  const int threads = 32 * (int)std::min<long>(G * NM * ngroup, 16);
  const size_t smem = (size_t)G * nn * sizeof(S) * (1 + NM) + sizeof(int) * (4 * ngroup + nrel);
  cudaError_t e = cudaFuncSetAttribute(k_minv_products<S, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_error(e, "k_minv_products");
  const long grid = std::min<long>((B + G - 1) / G, 152L * 8);
  for (int m0 = 0; m0 < 2; m0 += NM) {
    k_minv_products<S, W><<<(unsigned)grid, threads, smem, st>>>(M->d_blob, M->blob_bytes, B, (int)G, m0, NM, Minv, ws,
                                                             L.dtq, L.dtv, o0, o1);
    const int rc = cuda_error(cudaGetLastError(), "k_minv_products");
    if (rc != GB_OK) return rc;
  }
  return GB_OK;
}

template <class S>
int run_rnea_derivs(const gb_model* M, long B, bool symmetric, Arr q, Arr v, Arr a, Arr dq, Arr dv, Arr Mo, Arr tau,
                    cudaStream_t st) {
  const gb::DerivLayout L = gb::make_deriv_layout(M->nj, M->nv, M->nslot, false);
  Workspace ws;
  int rc = ws_alloc(ws, sizeof(S) * (size_t)L.nS * B, st);
  if (rc != GB_OK) return rc;
  rc = blob_smem(M, (const void*)k_rnea_derivs<S>, "k_rnea_derivs");
  if (rc != GB_OK) return rc;
  const int tpb = M->tpb[GB_FUNC_RNEA_DERIVATIVES];
  const long grid = (B + tpb - 1) / tpb;
  k_rnea_derivs<S><<<(unsigned)grid, tpb, M->blob_bytes, st>>>(M->d_blob, M->blob_bytes, B, L,
                                                                   static_cast<S*>(ws.p), symmetric, q, v, a, dq, dv,
                                                                   Mo, tau);
  return cuda_error(cudaGetLastError(), "k_rnea_derivs");
}

// Workspace of the ABA derivatives: region SS (FP64: kinematics, Schur, Minv
// data), region S (the derivative column passes: dfloat in the mixed kernels)
// and region P (dtau_dq, dtau_dv in the scalar of the -Minv*dtau products).
template <class S, class SS, class P>
size_t aba_ws_bytes(const gb::DerivLayout& L, long B) {
  return (sizeof(SS) * (size_t)L.nSS + sizeof(S) * (size_t)L.nS + sizeof(P) * (size_t)L.nP) * (size_t)B;
}

template <class S, class SS, class P>
int launch_aba_derivs_ws(const gb_model* M, long B, Arr q, Arr v, Arr tau, Arr dq, Arr dv, Arr Minv, Arr ddq, void* ws,
                         cudaStream_t st) {
  const gb::DerivLayout L = gb::make_deriv_layout(M->nj, M->nv, M->nslot, true);
  SS* wsSS = static_cast<SS*>(ws);
  S* wsS = reinterpret_cast<S*>(static_cast<char*>(ws) + sizeof(SS) * (size_t)L.nSS * B);
  P* wsP = reinterpret_cast<P*>(reinterpret_cast<char*>(wsS) + sizeof(S) * (size_t)L.nS * B);
  const int tpb = M->tpb[GB_FUNC_ABA_DERIVATIVES];
  const long grid = (B + tpb - 1) / tpb;
  int rc = blob_smem(M, (const void*)k_aba_derivs_pass12<S, SS>, "k_aba_derivs_pass12");
  if (rc == GB_OK) rc = blob_smem(M, (const void*)k_aba_derivs_pass3<S, SS>, "k_aba_derivs_pass3");
  if (rc == GB_OK) rc = blob_smem(M, (const void*)k_aba_derivs_pass4<S, SS, P>, "k_aba_derivs_pass4");
  if (rc != GB_OK) return rc;
  k_aba_derivs_pass12<S, SS><<<(unsigned)grid, tpb, M->blob_bytes, st>>>(M->d_blob, M->blob_bytes, B, L, wsSS, q, v,
                                                                             tau, Minv);
  rc = cuda_error(cudaGetLastError(), "k_aba_derivs_pass12");
  if (rc != GB_OK) return rc;
  k_aba_derivs_pass3<S, SS><<<(unsigned)grid, tpb, M->blob_bytes, st>>>(M->d_blob, M->blob_bytes, B, L, wsS, wsSS,
                                                                            v, Minv, ddq);
  rc = cuda_error(cudaGetLastError(), "k_aba_derivs_pass3");
  if (rc != GB_OK) return rc;
  k_aba_derivs_pass4<S, SS, P><<<(unsigned)grid, tpb, M->blob_bytes, st>>>(M->d_blob, M->blob_bytes, B, L, wsS,
                                                                               wsSS, wsP, Minv);
  rc = cuda_error(cudaGetLastError(), "k_aba_derivs_pass4");
  if (rc != GB_OK) return rc;
  return launch_minv_products<P, P>(M, B, Minv, wsP, L, dq, dv, st);
}

// S: scalar of the column passes (dfloat in the mixed kernels), SS: scalar of
// kinematics / Schur / Minv, P: scalar of the -Minv dtau products
template <class S, class SS, class P>
int run_aba_derivs(const gb_model* M, long B, Arr q, Arr v, Arr tau, Arr dq, Arr dv, Arr Minv, Arr ddq,
                   cudaStream_t st) {
  const gb::DerivLayout L = gb::make_deriv_layout(M->nj, M->nv, M->nslot, true);
  Workspace ws;
  int rc = ws_alloc(ws, aba_ws_bytes<S, SS, P>(L, B), st);
  if (rc != GB_OK) return rc;
  return launch_aba_derivs_ws<S, SS, P>(M, B, q, v, tau, dq, dv, Minv, ddq, ws.p, st);
}

int check_gravity(const gb_model* M) {
  if (M->gravity[3] != 0.0 || M->gravity[4] != 0.0 || M->gravity[5] != 0.0)
    return set_error(GB_ERR_GRAVITY, "The gravity must be a pure force vector, no angular part");
  return GB_OK;
}

}  // namespace

// The ABA-derivative kernels on a workspace the caller provides (no allocation):
// bytes needed per configuration, and the launch itself.
size_t aba_derivs_workspace_bytes(const gb_model* M, int precision) {
  const gb::DerivLayout L = gb::make_deriv_layout(M->nj, M->nv, M->nslot, true);
  return precision == GB_FP64 ? aba_ws_bytes<double, double, double>(L, 1) : aba_ws_bytes<gb::dfloat, double, float>(L, 1);
}

int launch_aba_derivs_on_workspace(const gb_model* M, int precision, long B, Arr q, Arr v, Arr tau, Arr dq, Arr dv,
                                   Arr Minv, Arr ddq, void* ws, cudaStream_t st) {
  if (check_gravity(M) != GB_OK) return GB_ERR_GRAVITY;
  if (precision == GB_FP64) return launch_aba_derivs_ws<double, double, double>(M, B, q, v, tau, dq, dv, Minv, ddq, ws, st);
  return launch_aba_derivs_ws<gb::dfloat, double, float>(M, B, q, v, tau, dq, dv, Minv, ddq, ws, st);
}

}  // namespace gbi

#define GB_TRY(x)                   \
  do {                              \
    const int rc__ = (x);           \
    if (rc__ != GB_OK) return rc__; \
  } while (0)

extern "C" {

int gb_rnea_derivatives(const gb_model* M, int precision, int matrix_mode, int layout, long B, const double* q,
                        const double* v, const double* a, double* dtau_dq, double* dtau_dv, double* Mo, double* tau,
                        void* stream) {
  GB_TRY(gbi::check_common(M, precision, layout, B));
  if (matrix_mode != GB_MATRIX_UPPER && matrix_mode != GB_MATRIX_SYMMETRIC)
    return gbi::set_error(GB_ERR_INVALID_ARGUMENT, "unknown matrix mode");
  GB_TRY(gbi::check_gravity(M));
  if (B == 0) return GB_OK;
  GB_TRY(gbi::check_ptr(q, "q")); GB_TRY(gbi::check_ptr(v, "v")); GB_TRY(gbi::check_ptr(a, "a"));
  GB_TRY(gbi::check_ptr(dtau_dq, "dtau_dq")); GB_TRY(gbi::check_ptr(dtau_dv, "dtau_dv")); GB_TRY(gbi::check_ptr(Mo, "M"));
  if (tau) GB_TRY(gbi::check_ptr(tau, "tau"));
  const long nn = (long)M->nv * M->nv;
  using gbi::arr;
  const gbi::Arr Aq = arr(q, layout, B, M->nq), Av = arr(v, layout, B, M->nv), Aa = arr(a, layout, B, M->nv);
  const gbi::Arr Adq = arr(dtau_dq, layout, B, nn), Adv = arr(dtau_dv, layout, B, nn), AM = arr(Mo, layout, B, nn);
  const gbi::Arr At = arr(tau, layout, B, M->nv);
  const bool sym = matrix_mode == GB_MATRIX_SYMMETRIC;
  cudaStream_t st = (cudaStream_t)stream;
  if (precision == GB_FP64) return gbi::run_rnea_derivs<double>(M, B, sym, Aq, Av, Aa, Adq, Adv, AM, At, st);
  return gbi::run_rnea_derivs<float>(M, B, sym, Aq, Av, Aa, Adq, Adv, AM, At, st);
}

int gb_aba_derivatives(const gb_model* M, int precision, int layout, long B, const double* q, const double* v,
                       const double* tau, double* ddq_dq, double* ddq_dv, double* Minv, double* ddq, void* stream) {
  GB_TRY(gbi::check_common(M, precision, layout, B));
  GB_TRY(gbi::check_gravity(M));
  if (B == 0) return GB_OK;
  GB_TRY(gbi::check_ptr(q, "q")); GB_TRY(gbi::check_ptr(v, "v")); GB_TRY(gbi::check_ptr(tau, "tau"));
  GB_TRY(gbi::check_ptr(ddq_dq, "ddq_dq")); GB_TRY(gbi::check_ptr(ddq_dv, "ddq_dv")); GB_TRY(gbi::check_ptr(Minv, "Minv"));
  if (ddq) GB_TRY(gbi::check_ptr(ddq, "ddq"));
  const long nn = (long)M->nv * M->nv;
  using gbi::arr;
  const gbi::Arr Aq = arr(q, layout, B, M->nq), Av = arr(v, layout, B, M->nv), At = arr(tau, layout, B, M->nv);
  const gbi::Arr Adq = arr(ddq_dq, layout, B, nn), Adv = arr(ddq_dv, layout, B, nn), AMi = arr(Minv, layout, B, nn);
  const gbi::Arr Add = arr(ddq, layout, B, M->nv);
  cudaStream_t st = (cudaStream_t)stream;
  if (precision == GB_FP64) return gbi::run_aba_derivs<double, double, double>(M, B, Aq, Av, At, Adq, Adv, AMi, Add, st);
  return gbi::run_aba_derivs<gb::dfloat, double, float>(M, B, Aq, Av, At, Adq, Adv, AMi, Add, st);
}

}  // extern "C"
