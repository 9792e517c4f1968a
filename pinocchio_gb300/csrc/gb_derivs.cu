// Batched analytical derivatives: computeRNEADerivatives and computeABADerivatives.
//
// RNEA derivatives: one kernel, one thread per configuration.
// ABA derivatives: (1) three sweep kernels (one thread per configuration) that
// produce ddq, Minv (packed upper triangle) and dtau_dq / dtau_dv at (q, v, ddq)
// in the workspace; (2) a CTA-cooperative kernel that writes the symmetric Minv
// and ddq_dq = -Minv dtau_dq, ddq_dv = -Minv dtau_dv (reference
// algorithm/aba-derivatives.hxx:451-452): G configurations are staged in shared
// memory, one warp owns one output matrix's column group, its lanes own rows,
// and for every column c the warp loops only over the rows k that can be
// non-zero in column c of dtau (ancestors and subtree of c) -- the reference
// multiplies the dense matrices.
#include "gb_derivs.cuh"
#include "gb_internal.h"

namespace gbi {
namespace {

constexpr int kThreads = 128;
// resident CTAs of kThreads per SM the derivative sweeps are compiled for (caps registers per thread)
#ifndef GB_DERIV_MINB
#define GB_DERIV_MINB 4
#endif

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
template <class K, class SS>
__global__ void __launch_bounds__(kThreads, GB_DERIV_MINB)
    k_aba_derivs_pass12(const unsigned char* blob, int bytes, long B, gb::DerivLayout L, K* wsK, SS* wsSS, Arr q,
                        Arr v, Arr tau) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_model(blob, bytes, smem);
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  gb::aba_derivs_pass12<K, SS>(m, L, gb::Ws<K>{wsK + b, B}, gb::Ws<SS>{wsSS + b, B}, in_at(q, b), in_at(v, b),
                               in_at(tau, b));
}

template <class S, class T, class K>
__global__ void __launch_bounds__(kThreads, GB_DERIV_MINB)
    k_aba_derivs_pass3(const unsigned char* blob, int bytes, long B, gb::DerivLayout L, S* wsS, K* wsK, Arr v,
                       Arr ddq) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_model(blob, bytes, smem);
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const gb::Out dd = out_at(ddq, b);
  gb::aba_derivs_pass3<S, T, K>(m, L, m.slot, gb::Ws<S>{wsS + b, B}, gb::Ws<K>{wsK + b, B}, in_at(v, b),
                                ddq.p ? &dd : nullptr);
}

template <class S, class T, class K, class P>
__global__ void __launch_bounds__(kThreads, GB_DERIV_MINB)
    k_aba_derivs_pass4(const unsigned char* blob, int bytes, long B, gb::DerivLayout L, S* wsS, K* wsK, P* wsP) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_model(blob, bytes, smem);
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  gb::aba_derivs_pass4<S, T, K, P>(m, L, gb::Ws<S>{wsS + b, B}, gb::Ws<K>{wsK + b, B}, gb::Ws<P>{wsP + b, B});
}

__device__ __forceinline__ double to_double(double x) { return x; }
__device__ __forceinline__ double to_double(float x) { return gb::widen(x); }
__device__ __forceinline__ double to_double(gb::dfloat x) { return double(x); }

// Minv and out_m = -Minv * X_m for the two matrices X_0 = dtau_dq, X_1 = dtau_dv
// of G consecutive configurations per iteration (G a power of two).  smem:
// Minv[G][nv*nv] (scalar S), then a region that first holds the packed upper
// Minv of the workspace (scalar KM) and then X[G][NM][nv*nv] (scalar S), then
// the column-group tables.  NM = number of the two products done per launch;
// the launch with m0 == 0 also writes the symmetric Minv output.  A warp owns
// one (configuration, matrix, column group); its lanes own rows (lane +
// 32*chunk, NCH chunks); for every row k that can be non-zero in the group's
// columns it loads one Minv row segment (lane-contiguous, Minv symmetric) and
// the group's <= 8 entries of X's row k (broadcast) and does up to 8 FMAs per
// lane.  With the instance layout each lane writes its row segment straight to
// the output; with the SoA layout the result goes back to X and is stored with
// the configurations contiguous.
template <int NCH, class S, class W, class KM>
__global__ void __launch_bounds__(512)
    k_minv_products(const unsigned char* blob, long B, int lgG, int m0, int NM, const KM* wsMi, Arr Minv,
                    const W* ws, long dtq, long dtv, Arr out0, Arr out1) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const gb::BlobHeader* h = reinterpret_cast<const gb::BlobHeader*>(blob);
  const int nv = h->nv, ng = h->ngroup, nrel = h->n_grp_rel;
  const int nn = nv * nv, npk = nv * (nv + 1) / 2;
  const int G = 1 << lgG;
  S* sM = reinterpret_cast<S*>(smem_raw);
  unsigned char* region = reinterpret_cast<unsigned char*>(sM + (long)G * nn);
  S* sX = reinterpret_cast<S*>(region);
  KM* sK = reinterpret_cast<KM*>(region);
  const size_t region_bytes = max((size_t)G * npk * sizeof(KM), (size_t)G * NM * nn * sizeof(S));
  int* sgrp = reinterpret_cast<int*>(region + ((region_bytes + 15) & ~(size_t)15));
  int* srel = sgrp + 4 * ng;
  for (int t = threadIdx.x; t < 4 * ng; t += blockDim.x) sgrp[t] = reinterpret_cast<const int*>(blob + h->o_grp)[t];
  for (int t = threadIdx.x; t < nrel; t += blockDim.x) srel[t] = reinterpret_cast<const int*>(blob + h->o_grp_rel)[t];
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32, nwarps = blockDim.x / 32;
  double* Mo = const_cast<double*>(Minv.p);
  for (long b0 = (long)blockIdx.x * G; b0 < B; b0 += (long)gridDim.x * G) {
    const int g_here = (int)min((long)G, B - b0);
    __syncthreads();
    // packed upper Minv of the workspace (SoA over the batch)
    for (int t = threadIdx.x; t < (npk << lgG); t += blockDim.x) {
      const int g = t & (G - 1), e = t >> lgG;
      if (g < g_here) sK[g * npk + e] = wsMi[(long)e * B + b0 + g];
    }
    __syncthreads();
    // full symmetric Minv: S copy for the products, FP64 output (launch m0 == 0)
    if (Minv.es == 1) {
      for (int g = 0; g < g_here; ++g) {
        double* dst = Mo + (b0 + g) * Minv.is;
        for (int e = threadIdx.x; e < nn; e += blockDim.x) {
          const int r = e / nv, c = e - r * nv;
          const KM x = sK[g * npk + (r <= c ? gb::upk(nv, r, c) : gb::upk(nv, c, r))];
          sM[g * nn + e] = S(x);
          if (m0 == 0) dst[e] = to_double(x);
        }
      }
    } else {
      for (int t = threadIdx.x; t < (nn << lgG); t += blockDim.x) {
        const int g = t & (G - 1), e = t >> lgG;
        if (g >= g_here) continue;
        const int r = e / nv, c = e - r * nv;
        const KM x = sK[g * npk + (r <= c ? gb::upk(nv, r, c) : gb::upk(nv, c, r))];
        sM[g * nn + e] = S(x);
        if (m0 == 0) Mo[(b0 + g) + (long)e * Minv.es] = to_double(x);
      }
    }
    __syncthreads();
    // the dtau matrices (workspace, SoA over the batch)
    for (int mm = 0; mm < NM; ++mm) {
      const W* src = ws + ((m0 + mm) == 0 ? dtq : dtv) * B + b0;
      for (int t = threadIdx.x; t < (nn << lgG); t += blockDim.x) {
        const int g = t & (G - 1), e = t >> lgG;
        if (g < g_here) sX[(g * NM + mm) * nn + e] = S(src[(long)e * B + g]);
      }
    }
    __syncthreads();
    const int ntask = g_here * NM * ng;
    for (int task = warp; task < ntask; task += nwarps) {
      const int g = task / (NM * ng), rem = task - g * (NM * ng), mm = rem / ng, gi = rem - mm * ng;
      const int c0 = sgrp[4 * gi], nc = sgrp[4 * gi + 1], k0 = sgrp[4 * gi + 2], k1 = sgrp[4 * gi + 3];
      const S* Mg = sM + g * nn;
      S* X = sX + (g * NM + mm) * nn;
      S acc[NCH][8];
#pragma unroll
      for (int ch = 0; ch < NCH; ++ch)
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
        for (int ch = 0; ch < NCH; ++ch) {
          const int r = ch * 32 + lane;
          const S mr = r < nv ? Mk[r] : S(0);
#pragma unroll
          for (int c = 0; c < 8; ++c) acc[ch][c] += mr * x[c];
        }
      }
      const Arr& o = (m0 + mm) == 0 ? out0 : out1;
      if (o.es == 1) {
        double* op = const_cast<double*>(o.p) + (b0 + g) * o.is + c0;
#pragma unroll
        for (int ch = 0; ch < NCH; ++ch) {
          const int r = ch * 32 + lane;
          if (r < nv)
#pragma unroll
            for (int c = 0; c < 8; ++c)
              if (c < nc) op[r * nv + c] = -to_double(acc[ch][c]);
        }
      } else {
        __syncwarp();
#pragma unroll
        for (int ch = 0; ch < NCH; ++ch) {
          const int r = ch * 32 + lane;
          if (r < nv)
#pragma unroll
            for (int c = 0; c < 8; ++c)
              if (c < nc) X[r * nv + c0 + c] = -acc[ch][c];
        }
        __syncwarp();
      }
    }
    __syncthreads();
    for (int mm = 0; mm < NM; ++mm) {
      const Arr& o = (m0 + mm) == 0 ? out0 : out1;
      if (o.es == 1) continue;
      double* op = const_cast<double*>(o.p) + b0;
      for (int t = threadIdx.x; t < (nn << lgG); t += blockDim.x) {
        const int g = t & (G - 1), e = t >> lgG;
        if (g < g_here) op[(long)e * o.es + g] = to_double(sX[(g * NM + mm) * nn + e]);
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

// S: scalar of the products (smem, FMA); W: scalar of the dtau matrices in the
// workspace; KM: scalar of the packed Minv in the workspace
template <int NCH, class S, class W, class KM>
int launch_minv_products_n(const gb_model* M, long B, const KM* wsMi, Arr Minv, const W* ws, const gb::DerivLayout& L,
                           Arr o0, Arr o1, cudaStream_t st) {
  const long nn = (long)M->nv * M->nv, npk = (long)M->nv * (M->nv + 1) / 2;
  const int ngroup = reinterpret_cast<const gb::BlobHeader*>(M->blob.data())->ngroup;
  const int nrel = reinterpret_cast<const gb::BlobHeader*>(M->blob.data())->n_grp_rel;
  auto smem_of = [&](long G, int NM) {
    const long region = std::max(G * npk * (long)sizeof(KM), G * NM * nn * (long)sizeof(S));
    return G * nn * (long)sizeof(S) + ((region + 15) & ~15L) + (long)sizeof(int) * (4 * ngroup + nrel);
  };
#ifndef GB_MINV_SMEM_KB
#define GB_MINV_SMEM_KB 100
#endif
  const long budget = GB_MINV_SMEM_KB * 1024;  // shared memory per CTA (100 KB: two CTAs per SM)
  int NM = 2, lgG = 3;
  while (lgG > 0 && smem_of(1L << lgG, NM) > budget) --lgG;
  if (smem_of(1L << lgG, NM) > budget) NM = 1;
  if (smem_of(1L << lgG, NM) > 220 * 1024) return set_error(GB_ERR_UNSUPPORTED, "nv too large for the Minv products");
  const long G = 1L << lgG;
  const int threads = 32 * (int)std::min<long>(G * NM * ngroup, 16);
  const size_t smem = (size_t)smem_of(G, NM);
  cudaError_t e =
      cudaFuncSetAttribute(k_minv_products<NCH, S, W, KM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_error(e, "k_minv_products");
  const long grid = std::min<long>((B + G - 1) / G, 152L * 2 * 8);
  for (int m0 = 0; m0 < 2; m0 += NM) {
    k_minv_products<NCH, S, W, KM><<<(unsigned)grid, threads, smem, st>>>(M->d_blob, B, lgG, m0, NM, wsMi, Minv, ws,
                                                                           L.dtq, L.dtv, o0, o1);
    const int rc = cuda_error(cudaGetLastError(), "k_minv_products");
    if (rc != GB_OK) return rc;
  }
  return GB_OK;
}

template <class S, class W, class KM>
int launch_minv_products(const gb_model* M, long B, const KM* wsMi, Arr Minv, const W* ws, const gb::DerivLayout& L,
                         Arr o0, Arr o1, cudaStream_t st) {
  if (M->nv <= 32) return launch_minv_products_n<1, S, W, KM>(M, B, wsMi, Minv, ws, L, o0, o1, st);
  if (M->nv <= 64) return launch_minv_products_n<2, S, W, KM>(M, B, wsMi, Minv, ws, L, o0, o1, st);
  return launch_minv_products_n<4, S, W, KM>(M, B, wsMi, Minv, ws, L, o0, o1, st);
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

// Workspace of the ABA derivatives: region SS (articulated inertias and u:
// FP64), region K (kinematics, Fcrb columns, Minv, U Dinv, Dinv u, velocity /
// acceleration), region S (the derivative column sets stored between passes 3
// and 4: computed in T3 by pass 3 and in T by pass 4) and region P (dtau_dq,
// dtau_dv in the scalar of the -Minv*dtau products).  The mixed kernels use
// K = T = dfloat, S = T3 = P = float.
template <class S, class T, class K, class SS, class P>
size_t aba_ws_bytes(const gb::DerivLayout& L, long B) {
  return (sizeof(SS) * (size_t)L.nSS + sizeof(K) * (size_t)L.nK + sizeof(S) * (size_t)L.nS +
          sizeof(P) * (size_t)L.nP) *
         (size_t)B;
}

template <class S, class T3, class T, class K, class SS, class P>
int launch_aba_derivs_ws(const gb_model* M, long B, Arr q, Arr v, Arr tau, Arr dq, Arr dv, Arr Minv, Arr ddq, void* ws,
                         cudaStream_t st) {
  const gb::DerivLayout L = gb::make_deriv_layout(M->nj, M->nv, M->nslot, true);
  SS* wsSS = static_cast<SS*>(ws);
  K* wsK = reinterpret_cast<K*>(static_cast<char*>(ws) + sizeof(SS) * (size_t)L.nSS * B);
  S* wsS = reinterpret_cast<S*>(reinterpret_cast<char*>(wsK) + sizeof(K) * (size_t)L.nK * B);
  P* wsP = reinterpret_cast<P*>(reinterpret_cast<char*>(wsS) + sizeof(S) * (size_t)L.nS * B);
  const int tpb = M->tpb[GB_FUNC_ABA_DERIVATIVES];
  const long grid = (B + tpb - 1) / tpb;
  int rc = blob_smem(M, (const void*)k_aba_derivs_pass12<K, SS>, "k_aba_derivs_pass12");
  if (rc == GB_OK) rc = blob_smem(M, (const void*)k_aba_derivs_pass3<S, T3, K>, "k_aba_derivs_pass3");
  if (rc == GB_OK) rc = blob_smem(M, (const void*)k_aba_derivs_pass4<S, T, K, P>, "k_aba_derivs_pass4");
  if (rc != GB_OK) return rc;
  k_aba_derivs_pass12<K, SS><<<(unsigned)grid, tpb, M->blob_bytes, st>>>(M->d_blob, M->blob_bytes, B, L, wsK, wsSS,
                                                                             q, v, tau);
  rc = cuda_error(cudaGetLastError(), "k_aba_derivs_pass12");
  if (rc != GB_OK) return rc;
  k_aba_derivs_pass3<S, T3, K><<<(unsigned)grid, tpb, M->blob_bytes, st>>>(M->d_blob, M->blob_bytes, B, L, wsS,
                                                                               wsK, v, ddq);
  rc = cuda_error(cudaGetLastError(), "k_aba_derivs_pass3");
  if (rc != GB_OK) return rc;
  k_aba_derivs_pass4<S, T, K, P><<<(unsigned)grid, tpb, M->blob_bytes, st>>>(M->d_blob, M->blob_bytes, B, L, wsS,
                                                                                 wsK, wsP);
  rc = cuda_error(cudaGetLastError(), "k_aba_derivs_pass4");
  if (rc != GB_OK) return rc;
  return launch_minv_products<P, P, K>(M, B, wsK + (long)L.Mi * B, Minv, wsP, L, dq, dv, st);
}

template <class S, class T3, class T, class K, class SS, class P>
int run_aba_derivs(const gb_model* M, long B, Arr q, Arr v, Arr tau, Arr dq, Arr dv, Arr Minv, Arr ddq,
                   cudaStream_t st) {
  const gb::DerivLayout L = gb::make_deriv_layout(M->nj, M->nv, M->nslot, true);
  Workspace ws;
  int rc = ws_alloc(ws, aba_ws_bytes<S, T, K, SS, P>(L, B), st);
  if (rc != GB_OK) return rc;
  return launch_aba_derivs_ws<S, T3, T, K, SS, P>(M, B, q, v, tau, dq, dv, Minv, ddq, ws.p, st);
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
  return precision == GB_FP64 ? aba_ws_bytes<double, double, double, double, double>(L, 1)
                              : aba_ws_bytes<float, gb::dfloat, gb::dfloat, double, float>(L, 1);
}

int launch_aba_derivs_on_workspace(const gb_model* M, int precision, long B, Arr q, Arr v, Arr tau, Arr dq, Arr dv,
                                   Arr Minv, Arr ddq, void* ws, cudaStream_t st) {
  if (check_gravity(M) != GB_OK) return GB_ERR_GRAVITY;
  if (precision == GB_FP64)
    return launch_aba_derivs_ws<double, double, double, double, double, double>(M, B, q, v, tau, dq, dv, Minv, ddq,
                                                                                ws, st);
  return launch_aba_derivs_ws<float, float, gb::dfloat, gb::dfloat, double, float>(M, B, q, v, tau, dq, dv, Minv, ddq,
                                                                                  ws, st);
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
  if (precision == GB_FP64)
    return gbi::run_aba_derivs<double, double, double, double, double, double>(M, B, Aq, Av, At, Adq, Adv, AMi, Add,
                                                                               st);
  return gbi::run_aba_derivs<float, float, gb::dfloat, gb::dfloat, double, float>(M, B, Aq, Av, At, Adq, Adv, AMi,
                                                                                 Add, st);
}

}  // extern "C"
