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

template <class S, class SS>
__global__ void __launch_bounds__(kThreads) k_aba_derivs_sweeps(const unsigned char* blob, int bytes, long B,
                                                                gb::DerivLayout L, S* wsS, SS* wsSS, Arr q, Arr v,
                                                                Arr tau, Arr Minv, Arr ddq) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_model(blob, bytes, smem);
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const gb::Ws<S> w{wsS + b, B};
  const gb::Ws<SS> z{wsSS + b, B};
  const gb::Out dd = out_at(ddq, b);
  gb::aba_derivs_sweeps<S, SS>(m, L, m.slot, w, z, in_at(q, b), in_at(v, b), in_at(tau, b), out_at(Minv, b),
                               ddq.p ? &dd : nullptr);
}

// out_m = -Minv * X_m for the two matrices X_0 = dtau_dq, X_1 = dtau_dv of G
// consecutive configurations per iteration.  smem: Minv[G][nv*nv] then
// X[G][NM][nv*nv] (scalar S).  NM = number of the two products done per pass.
template <class S, class W>
__global__ void k_minv_products(const unsigned char* blob, int bytes, long B, int G, int m0, int NM, Arr Minv,
                                const W* ws, long dtq, long dtv, Arr out0, Arr out1) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const gb::BlobHeader* h = reinterpret_cast<const gb::BlobHeader*>(blob);
  // the model blob is only needed for rel_off / rel_list: read them from global (L1-cached)
  const int nv = h->nv;
  const int* rel_off = reinterpret_cast<const int*>(blob + h->o_rel_off);
  const int* rel_list = reinterpret_cast<const int*>(blob + h->o_rel_list);
  const int nn = nv * nv;
  S* sM = reinterpret_cast<S*>(smem_raw);
  S* sX = sM + (long)G * nn;
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
    for (int task = warp; task < g_here * NM; task += nwarps) {
      const int g = task / NM, mm = task % NM;
      const S* Mg = sM + g * nn;
      S* X = sX + (g * NM + mm) * nn;
      for (int c = 0; c < nv; ++c) {
        const int k0 = rel_off[c], k1 = rel_off[c + 1];
        S acc[4] = {S(0), S(0), S(0), S(0)};  // rows lane, lane+32, lane+64, lane+96 (nv <= 128)
        for (int kk = k0; kk < k1; ++kk) {
          const int k = rel_list[kk];
          const S x = X[k * nv + c];
          const S* Mk = Mg + k * nv;  // Minv symmetric: Minv(r, k) = Minv(k, r)
#pragma unroll
          for (int ch = 0; ch < 4; ++ch) {
            const int r = ch * 32 + lane;
            if (r < nv) acc[ch] += Mk[r] * x;
          }
        }
        __syncwarp();
        // column c of X is no longer read: store the result column there
#pragma unroll
        for (int ch = 0; ch < 4; ++ch) {
          const int r = ch * 32 + lane;
          if (r < nv) X[r * nv + c] = -acc[ch];
        }
        __syncwarp();
      }
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
  const long budget = 200 * 1024;
  int NM = 2;
  long G = budget / (nn * (long)sizeof(S) * (1 + NM));
  if (G < 1) {
    NM = 1;
    G = budget / (nn * (long)sizeof(S) * (1 + NM));
  }
  if (G < 1) return set_error(GB_ERR_UNSUPPORTED, "nv too large for the Minv products");
  G = std::min<long>(G, 16);
  const int threads = 32 * (int)std::min<long>(G * NM, 16);
  const size_t smem = (size_t)G * nn * sizeof(S) * (1 + NM);
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
  const long grid = (B + kThreads - 1) / kThreads;
  k_rnea_derivs<S><<<(unsigned)grid, kThreads, M->blob_bytes, st>>>(M->d_blob, M->blob_bytes, B, L,
                                                                   static_cast<S*>(ws.p), symmetric, q, v, a, dq, dv,
                                                                   Mo, tau);
  return cuda_error(cudaGetLastError(), "k_rnea_derivs");
}

// S: scalar of the FP32-side derivative passes (dfloat in the mixed kernels),
// SS: scalar of kinematics / Schur / Minv, P: scalar of the -Minv dtau products
template <class S, class SS, class P>
int run_aba_derivs(const gb_model* M, long B, Arr q, Arr v, Arr tau, Arr dq, Arr dv, Arr Minv, Arr ddq,
                   cudaStream_t st) {
  const gb::DerivLayout L = gb::make_deriv_layout(M->nj, M->nv, M->nslot, true);
  const size_t bSS = sizeof(SS) * (size_t)L.nSS * B;
  const size_t bS = sizeof(S) * (size_t)L.nS * B;
  Workspace ws;
  int rc = ws_alloc(ws, bSS + bS, st);
  if (rc != GB_OK) return rc;
  SS* wsSS = static_cast<SS*>(ws.p);
  S* wsS = reinterpret_cast<S*>(static_cast<char*>(ws.p) + bSS);
  rc = blob_smem(M, (const void*)k_aba_derivs_sweeps<S, SS>, "k_aba_derivs_sweeps");
  if (rc != GB_OK) return rc;
  const long grid = (B + kThreads - 1) / kThreads;
  k_aba_derivs_sweeps<S, SS><<<(unsigned)grid, kThreads, M->blob_bytes, st>>>(M->d_blob, M->blob_bytes, B, L, wsS,
                                                                             wsSS, q, v, tau, Minv, ddq);
  rc = cuda_error(cudaGetLastError(), "k_aba_derivs_sweeps");
  if (rc != GB_OK) return rc;
  return launch_minv_products<P, S>(M, B, Minv, wsS, L, dq, dv, st);
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
  const size_t s = precision == GB_FP64 ? sizeof(double) : sizeof(gb::dfloat);
  return sizeof(double) * (size_t)L.nSS + s * (size_t)L.nS;
}

int launch_aba_derivs_on_workspace(const gb_model* M, int precision, long B, Arr q, Arr v, Arr tau, Arr dq, Arr dv,
                                   Arr Minv, Arr ddq, void* ws, cudaStream_t st) {
  if (check_gravity(M) != GB_OK) return GB_ERR_GRAVITY;
  const gb::DerivLayout L = gb::make_deriv_layout(M->nj, M->nv, M->nslot, true);
  const long grid = (B + kThreads - 1) / kThreads;
  const size_t bSS = sizeof(double) * (size_t)L.nSS * B;
  double* wsSS = static_cast<double*>(ws);
  if (precision == GB_FP64) {
    double* wsS = reinterpret_cast<double*>(static_cast<char*>(ws) + bSS);
    int rc = blob_smem(M, (const void*)k_aba_derivs_sweeps<double, double>, "k_aba_derivs_sweeps");
    if (rc != GB_OK) return rc;
    k_aba_derivs_sweeps<double, double><<<(unsigned)grid, kThreads, M->blob_bytes, st>>>(
        M->d_blob, M->blob_bytes, B, L, wsS, wsSS, q, v, tau, Minv, ddq);
    rc = cuda_error(cudaGetLastError(), "k_aba_derivs_sweeps");
    if (rc != GB_OK) return rc;
    return launch_minv_products<double, double>(M, B, Minv, wsS, L, dq, dv, st);
  }
  gb::dfloat* wsS = reinterpret_cast<gb::dfloat*>(static_cast<char*>(ws) + bSS);
  int rc = blob_smem(M, (const void*)k_aba_derivs_sweeps<gb::dfloat, double>, "k_aba_derivs_sweeps");
  if (rc != GB_OK) return rc;
  k_aba_derivs_sweeps<gb::dfloat, double><<<(unsigned)grid, kThreads, M->blob_bytes, st>>>(
      M->d_blob, M->blob_bytes, B, L, wsS, wsSS, q, v, tau, Minv, ddq);
  rc = cuda_error(cudaGetLastError(), "k_aba_derivs_sweeps");
  if (rc != GB_OK) return rc;
  return launch_minv_products<float, gb::dfloat>(M, B, Minv, wsS, L, dq, dv, st);
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
