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
#include <algorithm>
#include <type_traits>
#include <vector>

#include "gb_async.cuh"
#include "gb_sweeps.cuh"

namespace gbi {
namespace {

// FE: with external forces (fext, njoints x 6 per configuration in the joint frames)
template <class S, bool FE = false, bool J3 = false>
__global__ void __launch_bounds__(kThreads) k_rnea_derivs(const unsigned char* blob, int bytes, long B,
                                                          gb::DerivLayout L, S* ws, bool symmetric, Arr q, Arr v,
                                                          Arr a, Arr dq, Arr dv, Arr Mo, Arr tau, Arr fext) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_model(blob, bytes, smem);
  const long b = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= B) return;
  const gb::Ws<S> w{ws + b, B};
  const gb::Out to = out_at(tau, b);
  const gb::In fe = in_at(fext, b);
  gb::rnea_derivs_one<S, J3>(m, L, w, in_at(q, b), in_at(v, b), in_at(a, b), out_at(dq, b), out_at(dv, b), out_at(Mo, b),
                         tau.p ? &to : nullptr, symmetric, true, FE ? &fe : nullptr);
}

__device__ __forceinline__ double to_double(double x) { return x; }
__device__ __forceinline__ double to_double(float x) { return gb::widen(x); }
__device__ __forceinline__ double to_double(gb::dfloat x) { return double(x); }


// Minv and out_m = -Minv * X_m for the two matrices X_0 = dtau_dq, X_1 = dtau_dv.
// A CTA iteration takes Gs = 2^lgG (<= kBlk) configurations of one block; shared
// memory holds them interleaved ([element][configuration]): the full Minv
// (scalar S), then a region that first holds the packed upper Minv (scalar KM)
// and then X for NM of the two matrices (scalar S), then the column-group
// tables.  The launch with m0 == 0 also writes the symmetric Minv output.  A
// warp task is (matrix, column group, 64 / Gs rows); lane = (row pair,
// config), so the Minv and X reads are conflict-free; for every row k that
// can be non-zero in the group's columns a lane loads two Minv entries and the
// group's <= 8 entries of X's row k and does 16 FMAs; each lane writes its two
// row segments.
template <int LG, class S, class W, class KM>
__global__ void __launch_bounds__(512, 2)
    k_minv_products(const unsigned char* blob, long B, int m0, int NM, const KM* wsMi, Arr Minv, bool minv_upper,
                    const W* wsP, long nP, long dtq, long dtv, Arr out0, Arr out1) {
  constexpr int Gs = 1 << LG, R = 32 >> LG;  // configurations per iteration, rows per warp task
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const gb::BlobHeader* h = reinterpret_cast<const gb::BlobHeader*>(blob);
  const int nv = h->nv, ng = h->ngroup, nrel = h->n_grp_rel;
  const int nn = nv * nv, npk = nv * (nv + 1) / 2;
  S* sM = reinterpret_cast<S*>(smem_raw);
  unsigned char* region = reinterpret_cast<unsigned char*>(sM + (long)nn * Gs);
  S* sX = reinterpret_cast<S*>(region);
  KM* sK = reinterpret_cast<KM*>(region);
  const size_t region_bytes = max((size_t)npk * Gs * sizeof(KM), ((size_t)NM * nn + 8) * Gs * sizeof(S));
  int* sgrp = reinterpret_cast<int*>(region + ((region_bytes + 15) & ~(size_t)15));
  int* srel = sgrp + 4 * ng;
  for (int t = threadIdx.x; t < 4 * ng; t += blockDim.x) sgrp[t] = reinterpret_cast<const int*>(blob + h->o_grp)[t];
  for (int t = threadIdx.x; t < nrel; t += blockDim.x) srel[t] = reinterpret_cast<const int*>(blob + h->o_grp_rel)[t];
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32, nwarps = blockDim.x / 32;
  const int lr = lane >> LG, lg = lane & (Gs - 1);  // lane's row in the task, lane's configuration
  const long nblk = (B + kBlk - 1) / kBlk, nit = nblk << (3 - LG);
  double* Mo = const_cast<double*>(Minv.p);
  const int nrc = (nv + R - 1) / R;        // row chunks of the Minv expansion
  const int nrt = (nv + 2 * R - 1) / (2 * R);  // row chunks of the products: two rows per lane
  const int rowstride = nv * Gs;           // between rows k of one matrix in shared memory
  for (long it = blockIdx.x; it < nit; it += gridDim.x) {
    const long blk = it >> (3 - LG);
    const int g0 = (int)(it & ((kBlk >> LG) - 1)) << LG;
    const long b0 = blk * kBlk + g0;
    if (b0 >= B) continue;
    const int g_here = (int)min((long)Gs, B - b0);
    __syncthreads();
    // packed upper Minv of the iteration's configurations (contiguous when Gs == kBlk)
    {
      const KM* src = wsMi + blk * (long)npk * kBlk + g0;
      auto at = [&](int t) { return Gs == kBlk ? src[t] : src[(long)(t >> LG) * kBlk + (t & (Gs - 1))]; };
      const int n = npk << LG, step = blockDim.x;
      int t = threadIdx.x;
      for (; t + 3 * step < n; t += 4 * step) {  // four loads in flight per thread
        const KM a0 = at(t), a1 = at(t + step), a2 = at(t + 2 * step), a3 = at(t + 3 * step);
        sK[t] = a0; sK[t + step] = a1; sK[t + 2 * step] = a2; sK[t + 3 * step] = a3;
      }
      for (; t < n; t += step) sK[t] = at(t);
    }
    __syncthreads();
    // full symmetric Minv: S copy for the products, FP64 output (launch m0 == 0).
    // A warp covers (row r, 32 / Gs columns) x Gs configurations.
    for (int rc = warp; rc < nv * nrc; rc += nwarps) {
      const int r = rc / nrc, c = (rc - r * nrc) * R + lr;
      if (c >= nv) continue;
      const KM x = sK[(r <= c ? gb::upk(nv, r, c) : gb::upk(nv, c, r)) * Gs + lg];
      sM[(r * nv + c) * Gs + lg] = S(x);
      if (m0 == 0 && lg < g_here)
        Mo[(b0 + lg) * Minv.is + (long)(r * nv + c) * Minv.es] = (minv_upper && r > c) ? 0.0 : to_double(x);
    }
    __syncthreads();
    if (NM == 0) continue;  // Minv only
    // the dtau matrices
    for (int mm = 0; mm < NM; ++mm) {
      const W* src = wsP + blk * nP * kBlk + ((m0 + mm) == 0 ? dtq : dtv) * kBlk + g0;
      S* dst = sX + (long)mm * nn * Gs;
      auto at = [&](int t) { return S(Gs == kBlk ? src[t] : src[(long)(t >> LG) * kBlk + (t & (Gs - 1))]); };
      const int n = nn << LG, step = blockDim.x;
      int t = threadIdx.x;
      for (; t + 3 * step < n; t += 4 * step) {
        const S a0 = at(t), a1 = at(t + step), a2 = at(t + 2 * step), a3 = at(t + 3 * step);
        dst[t] = a0; dst[t + step] = a1; dst[t + 2 * step] = a2; dst[t + 3 * step] = a3;
      }
      for (; t < n; t += step) dst[t] = at(t);
    }
    __syncthreads();
    const int ntask = NM * ng * nrt;
    for (int task = warp; task < ntask; task += nwarps) {
      const int mm = task / (ng * nrt), rem = task - mm * (ng * nrt), gi = rem / nrt, rch = rem - gi * nrt;
      const int r0 = rch * 2 * R + lr, r1 = r0 + R;
      const int c0 = sgrp[4 * gi], nc = sgrp[4 * gi + 1], k0 = sgrp[4 * gi + 2], k1 = sgrp[4 * gi + 3];
      const S* Xg = sX + ((long)mm * nn + c0) * Gs + lg;
      const S* M0 = sM + (r0 < nv ? r0 : 0) * Gs + lg;
      const S* M1 = sM + (r1 < nv ? r1 : 0) * Gs + lg;
      S acc0[8], acc1[8];
#pragma unroll
      for (int c = 0; c < 8; ++c) acc0[c] = acc1[c] = S(0);
#pragma unroll 2
      for (int kk = k0; kk < k1; ++kk) {
        const int ko = srel[kk] * rowstride;
        const S m0v = M0[ko], m1v = M1[ko];  // Minv(k, r) = Minv(r, k)
        const S* Xk = Xg + ko;
#pragma unroll
        for (int c = 0; c < 8; ++c) {  // past the group: padded, not stored
          const S x = Xk[c * Gs];
          acc0[c] += m0v * x;
          acc1[c] += m1v * x;
        }
      }
      if (lg >= g_here) continue;
      const Arr& o = (m0 + mm) == 0 ? out0 : out1;
      double* ob = const_cast<double*>(o.p) + (b0 + lg) * o.is + (long)c0 * o.es;
#pragma unroll
      for (int h2 = 0; h2 < 2; ++h2) {
        const int r = h2 == 0 ? r0 : r1;
        if (r >= nv) continue;
        double* op = ob + (long)r * nv * o.es;
        if (o.es == 1) {
#pragma unroll
          for (int c = 0; c < 8; ++c)
            if (c < nc) op[c] = -to_double(h2 == 0 ? acc0[c] : acc1[c]);
        } else {
#pragma unroll
          for (int c = 0; c < 8; ++c)
            if (c < nc) op[c * o.es] = -to_double(h2 == 0 ? acc0[c] : acc1[c]);
        }
      }
    }
  }
}

// The mixed-precision products as a warp-specialised pipeline: one persistent
// CTA per SM walks the blocks of kBlk configurations with two stages.
//  - Producer warps (GB_PROD_PWARPS): for block j they wait until stage j % 2
//    is free, let the TMA unit copy both dtau matrices of the block (FP32,
//    already in the [element][configuration] order the FMA loop reads) into
//    the stage with one bulk copy completing on full_x, read the packed upper
//    Minv (double-float) with coalesced loads, write the FP64 Minv output and
//    the full FP32 Minv of the stage, and arrive on full_m.
//  - Consumer warps (GB_PROD_CWARPS): wait on full_x and full_m, run the
//    column-group products of k_minv_products with four output rows per lane
//    (Minv kept as [k][row / 4][configuration][row % 4]: one 16-byte load gives
//    a lane its four Minv(k, row), each X(k, c) read feeds four FMAs), write the
//    outputs and arrive on empty.  Warp tasks (matrix, column group, 16 rows)
//    are assigned in longest-processing-time order (ProdPlan).
// The producers fill block j + 1 while the consumers work on block j; no CTA-wide
// barrier after the start.  Every wait gives up after kPipeWaitNs (counted in
// g_pipe_timeouts).  Same FP32 products and summation order as k_minv_products:
// the outputs are bit-identical to k_minv_products<3, float, float, dfloat>.
#ifndef GB_PROD_CWARPS
#define GB_PROD_CWARPS 12
#endif
#ifndef GB_PROD_PWARPS
#define GB_PROD_PWARPS 4
#endif
constexpr int kProdMaxWarps = 32, kProdMaxTasks = 256, kProdRows = 16;  // rows per task (4 per lane)
struct ProdPlan {
  unsigned short woff[kProdMaxWarps + 1];  // consumer warp w runs task[woff[w] .. woff[w+1])
  unsigned short task[kProdMaxTasks];      // matrix | group << 1 | row chunk << 8
};
static_assert(sizeof(ProdPlan::woff) == sizeof(gb_model::prod_woff) &&
                  sizeof(ProdPlan::task) == sizeof(gb_model::prod_task),
              "the model caches the product plan");
__device__ unsigned int g_pipe_timeouts = 0;  // warps whose pipeline wait gave up (gb_pipeline_timeouts)
constexpr unsigned long long kPipeWaitNs = 2000000000ull;

struct PipeSmem {
  size_t oK, oX0, oX1, oM0, oM1, oT, bytes;
};
__host__ __device__ __forceinline__ PipeSmem pipe_smem(int nv, int ng, int nrel) {
  const size_t nn = (size_t)nv * nv, npk = (size_t)nv * (nv + 1) / 2;
  PipeSmem p;
  p.oK = 64;  // seven mbarriers first
  p.oX0 = p.oK + ((npk * kBlk * sizeof(gb::dfloat) + 15) & ~(size_t)15);
  p.oX1 = p.oX0 + 2 * nn * kBlk * sizeof(float);
  p.oM0 = p.oX1 + 2 * nn * kBlk * sizeof(float);
  p.oM1 = p.oM0 + nn * kBlk * sizeof(float);
  p.oT = p.oM1 + nn * kBlk * sizeof(float);
  p.bytes = p.oT + sizeof(int) * (4 * (size_t)ng + nrel);
  return p;
}

__global__ void __launch_bounds__((GB_PROD_CWARPS + GB_PROD_PWARPS) * 32, 1)
    k_minv_products_pipe(const unsigned char* blob, long B, const gb::dfloat* wsMi, Arr Minv, bool minv_upper,
                         const float* wsP, long nP, Arr out0, Arr out1, const __grid_constant__ ProdPlan plan) {
  constexpr int Gs = kBlk, CW = GB_PROD_CWARPS, PW = GB_PROD_PWARPS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const gb::BlobHeader* h = reinterpret_cast<const gb::BlobHeader*>(blob);
  const int nv = h->nv, ng = h->ngroup, nrel = h->n_grp_rel;
  const int nn = nv * nv, npk = nv * (nv + 1) / 2;
  const PipeSmem P = pipe_smem(nv, ng, nrel);
  uint64_t* full_x = reinterpret_cast<uint64_t*>(smem_raw);  // [2]: the stage's dtau copy landed
  uint64_t* full_m = full_x + 2;                             // [2]: the stage's FP32 Minv is written
  uint64_t* empty = full_x + 4;                              // [2]: the consumers are done with the stage
  uint64_t* full_k = full_x + 6;                             // the packed Minv copy landed (one buffer)
  gb::dfloat* sK = reinterpret_cast<gb::dfloat*>(smem_raw + P.oK);
  float* const sX0 = reinterpret_cast<float*>(smem_raw + P.oX0);
  float* const sX1 = reinterpret_cast<float*>(smem_raw + P.oX1);
  float* const sM0 = reinterpret_cast<float*>(smem_raw + P.oM0);
  float* const sM1 = reinterpret_cast<float*>(smem_raw + P.oM1);
  int* sgrp = reinterpret_cast<int*>(smem_raw + P.oT);
  int* srel = sgrp + 4 * ng;
  const uint32_t bytesX = 2u * nn * Gs * sizeof(float), bytesK = (uint32_t)npk * Gs * sizeof(gb::dfloat);
  const long nblk = (B + kBlk - 1) / kBlk;
  if (threadIdx.x == 0) {
    for (int s = 0; s < 2; ++s) {
      gb::mbar_init(&full_x[s], 1);
      gb::mbar_init(&full_m[s], PW * 32);
      gb::mbar_init(&empty[s], CW * 32);
    }
    gb::mbar_init(full_k, 1);
    gb::fence_mbar_init();
  }
  for (int t = threadIdx.x; t < 4 * ng; t += blockDim.x) sgrp[t] = reinterpret_cast<const int*>(blob + h->o_grp)[t];
  for (int t = threadIdx.x; t < nrel; t += blockDim.x) srel[t] = reinterpret_cast<const int*>(blob + h->o_grp_rel)[t];
  __syncthreads();
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int lg = lane & (Gs - 1);
  auto give_up = [&]() {
    if (lane == 0) atomicAdd(&g_pipe_timeouts, 1u);
  };
  if (warp >= CW) {  // ---------------- producers
    const int pt = threadIdx.x - CW * 32, pw = warp - CW, lr = lane >> 3;
    double* Mo = const_cast<double*>(Minv.p);
    auto load_minv = [&](long blk) {
      gb::mbar_arrive_expect_tx(full_k, bytesK);
      gb::bulk_load(sK, wsMi + blk * (long)npk * Gs, bytesK, full_k);
    };
    if (pt == 0 && blockIdx.x < nblk) load_minv(blockIdx.x);
    int j = 0;
    for (long blk = blockIdx.x; blk < nblk; blk += gridDim.x, ++j) {
      const int s = j & 1;
      const uint32_t n = (uint32_t)(j >> 1);
      bool ok = j < 2 || gb::mbar_wait(&empty[s], (n - 1) & 1u, kPipeWaitNs);
      ok = gb::named_bar_all(1, PW * 32, ok);  // the same decision in every producer thread
      if (ok && pt == 0) {
        gb::fence_proxy_async();
        gb::mbar_arrive_expect_tx(&full_x[s], bytesX);
        gb::bulk_load(s ? sX1 : sX0, wsP + blk * nP * Gs, bytesX, &full_x[s]);
      }
      const bool issued_x = ok;
      ok = gb::named_bar_all(1, PW * 32, ok && gb::mbar_wait(full_k, (uint32_t)j & 1u, kPipeWaitNs));
      if (!ok) {
        if (pt == 0) {  // let the copies this thread issued finish before leaving
          gb::mbar_wait(full_k, (uint32_t)j & 1u, kPipeWaitNs);
          if (issued_x) gb::mbar_wait(&full_x[s], n & 1u, kPipeWaitNs);
          if (j >= 1) gb::mbar_wait(&full_x[s ^ 1], ((uint32_t)(j - 1) >> 1) & 1u, kPipeWaitNs);
        }
        give_up();
        return;
      }
      float* sM = s ? sM1 : sM0;
      const long b0 = blk * kBlk;
      const int g_here = (int)min((long)Gs, B - b0);
      double* ob = Mo + (b0 + lg) * Minv.is;
      // one packed entry (a <= b) per lane step; producer warp t takes rows t, nv - 1 - t, t + PW, ...
      for (int t = pw; 2 * t < nv; t += PW) {
#pragma unroll 1
        for (int h2 = 0; h2 < 2; ++h2) {
          const int a = h2 == 0 ? t : nv - 1 - t;
          if (h2 == 1 && a == t) break;
          const int pa = a * nv - (a * (a - 1)) / 2 - a;  // upk(a, b) = pa + b for b >= a
          for (int b = a + lr; b < nv; b += 4) {
            const gb::dfloat x = sK[(pa + b) * Gs + lg];
            const float xf = float(x);
            sM[(a * nv + b) * Gs + lg] = xf;
            sM[(b * nv + a) * Gs + lg] = xf;
            if (lg < g_here) {
              const double xd = to_double(x);
              ob[(long)(a * nv + b) * Minv.es] = xd;
              ob[(long)(b * nv + a) * Minv.es] = minv_upper && b > a ? 0.0 : xd;
            }
          }
        }
      }
      gb::named_bar(1, PW * 32);  // all producers are done with sK
      const long nxt = blk + gridDim.x;
      if (pt == 0 && nxt < nblk) {
        gb::fence_proxy_async();
        load_minv(nxt);
      }
      gb::mbar_arrive(&full_m[s]);
    }
    return;
  }
  // ---------------- consumers
  // lane = (configuration quad cq, column c_l, row r_l): configurations 4 cq .. 4 cq + 3, columns c_l and
  // c_l + 4 of the group, rows r_l + 4 i (i < 4) of the task's 16; every shared load is 16 bytes (four
  // configurations) and the 32 lanes' addresses fall in distinct banks
  const int cq = lane >> 4, cl = (lane >> 2) & 3, rl = lane & 3;
  int j = 0;
  for (long blk = blockIdx.x; blk < nblk; blk += gridDim.x, ++j) {
    const int s = j & 1;
    const uint32_t par = (uint32_t)(j >> 1) & 1u;
    if (!gb::mbar_wait(&full_x[s], par, kPipeWaitNs) || !gb::mbar_wait(&full_m[s], par, kPipeWaitNs)) {
      give_up();
      return;
    }
    const long b0 = blk * kBlk;
    const int g_here = (int)min((long)Gs, B - b0);
    const float* sX = s ? sX1 : sX0;
    const float* sM = s ? sM1 : sM0;
    for (int p = plan.woff[warp]; p < plan.woff[warp + 1]; ++p) {
      const int task = plan.task[p];
      const int mm = task & 1, gi = (task >> 1) & 127, rch = task >> 8;
      const int c0 = sgrp[4 * gi], nc = sgrp[4 * gi + 1], k0 = sgrp[4 * gi + 2], k1 = sgrp[4 * gi + 3];
      const int r0 = rch * kProdRows + rl;  // the lane's rows: r0 + 4 i
      const float* Xg = sX + ((long)mm * nn + c0 + cl) * Gs + 4 * cq;
      const float* Mr[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) Mr[i] = sM + min(r0 + 4 * i, nv - 1) * Gs + 4 * cq;  // rows past nv: not stored
      float acc[4][2][4];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int cc = 0; cc < 2; ++cc)
#pragma unroll
          for (int g = 0; g < 4; ++g) acc[i][cc][g] = 0.f;
#pragma unroll 2
      for (int kk = k0; kk < k1; ++kk) {
        const int kb = srel[kk] * nv * Gs;
        const float4 x0 = *reinterpret_cast<const float4*>(Xg + kb);  // X(k, c_l), X(k, c_l + 4): past the group
        const float4 x1 = *reinterpret_cast<const float4*>(Xg + kb + 4 * Gs);  // padded, not stored
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const float4 m = *reinterpret_cast<const float4*>(Mr[i] + kb);  // Minv(k, r) = Minv(r, k)
          acc[i][0][0] += m.x * x0.x; acc[i][0][1] += m.y * x0.y; acc[i][0][2] += m.z * x0.z; acc[i][0][3] += m.w * x0.w;
          acc[i][1][0] += m.x * x1.x; acc[i][1][1] += m.y * x1.y; acc[i][1][2] += m.z * x1.z; acc[i][1][3] += m.w * x1.w;
        }
      }
      const Arr& o = mm == 0 ? out0 : out1;
      double* ob = const_cast<double*>(o.p) + (b0 + 4 * cq) * o.is + (long)(c0 + cl) * o.es;
      const bool st0 = cl < nc, st1 = cl + 4 < nc;
      if (o.es == 1 && g_here == Gs && r0 + 12 < nv) {  // the common case: predicated stores only
#pragma unroll
        for (int g = 0; g < 4; ++g)
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            double* op = ob + g * o.is + (r0 + 4 * i) * nv;
            if (st0) op[0] = to_double(-acc[i][0][g]);
            if (st1) op[4] = to_double(-acc[i][1][g]);
          }
      } else {
#pragma unroll
        for (int g = 0; g < 4; ++g) {
          if (4 * cq + g >= g_here) break;
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const int r = r0 + 4 * i;
            if (r >= nv) break;
            double* op = ob + g * o.is + (long)r * nv * o.es;
            if (st0) op[0] = to_double(-acc[i][0][g]);
            if (st1) op[4 * o.es] = to_double(-acc[i][1][g]);
          }
        }
      }
    }
    gb::mbar_arrive(&empty[s]);
  }
}

// The bounded wait's failure path, exercised without a fault: one warp waits on an
// mbarrier that nothing arrives on, gives up after limit_ns and records the timeout
// exactly as the pipeline's warps do.
__global__ void k_wait_selftest(unsigned long long limit_ns) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    gb::mbar_init(&bar, 1);
    gb::fence_mbar_init();
  }
  __syncwarp();
  const bool ok = gb::mbar_wait(&bar, 0u, limit_ns);
  if (!__any_sync(0xffffffffu, ok) && threadIdx.x == 0) atomicAdd(&g_pipe_timeouts, 1u);
}

// Longest-processing-time assignment of the product tasks to nwarps warps.
bool make_prod_plan(const gb_model* M, int nwarps, ProdPlan& plan) {
  const gb::BlobHeader* h = reinterpret_cast<const gb::BlobHeader*>(M->blob.data());
  const int* grp = reinterpret_cast<const int*>(M->blob.data() + h->o_grp);
  const int ng = h->ngroup, nrt = (M->nv + kProdRows - 1) / kProdRows, nt = 2 * ng * nrt;
  if (nt > kProdMaxTasks || nwarps > kProdMaxWarps || ng > 127 || nrt > 127) return false;
  std::vector<std::pair<int, int>> tasks;  // (cost, task)
  for (int mm = 0; mm < 2; ++mm)
    for (int gi = 0; gi < ng; ++gi)
      for (int rch = 0; rch < nrt; ++rch) tasks.push_back({grp[4 * gi + 3] - grp[4 * gi + 2] + 2, mm | gi << 1 | rch << 8});
  std::stable_sort(tasks.begin(), tasks.end(), [](auto a, auto b) { return a.first > b.first; });
  std::vector<long> load(nwarps, 0);
  std::vector<std::vector<int>> per(nwarps);
  for (const auto& ct : tasks) {
    const int w = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    load[w] += ct.first;
    per[w].push_back(ct.second);
  }
  int p = 0;
  for (int w = 0; w <= kProdMaxWarps; ++w) {
    plan.woff[w] = (unsigned short)p;
    if (w < nwarps) for (int t : per[w]) plan.task[p++] = (unsigned short)t;
  }
  return true;
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
  return scratch_alloc(&w.p, bytes, st);
}

#ifndef GB_PROD_PIPE
#define GB_PROD_PIPE 1
#endif
// the pipelined mixed products when the two stages fit in one CTA's shared
// memory (nv <= 32); used == false leaves the call to k_minv_products
int launch_products_pipe(const gb_model* M, long B, const gb::dfloat* wsMi, Arr Minv, bool minv_upper,
                         const float* wsP, long nP, Arr o0, Arr o1, cudaStream_t st, bool& used) {
  used = false;
  if (!GB_PROD_PIPE || !M->prod_plan_ok) return GB_OK;  // plan and shared-memory size: set at model creation
  const gb::BlobHeader* h = reinterpret_cast<const gb::BlobHeader*>(M->blob.data());
  const PipeSmem P = pipe_smem(M->nv, h->ngroup, h->n_grp_rel);
  ProdPlan plan;
  std::copy(M->prod_woff, M->prod_woff + kProdMaxWarps + 1, plan.woff);
  std::copy(M->prod_task, M->prod_task + kProdMaxTasks, plan.task);
  const long nblk = (B + kBlk - 1) / kBlk;
  const long grid = std::min<long>(nblk, M->sm_count);
  k_minv_products_pipe<<<(unsigned)grid, (GB_PROD_CWARPS + GB_PROD_PWARPS) * 32, P.bytes, st>>>(M->d_blob, B, wsMi, Minv, minv_upper, wsP,
                                                                          nP, o0, o1, plan);
  used = true;
  return cuda_error(cudaGetLastError(), "k_minv_products_pipe");
}

// S: scalar of the products (smem, FMA); W: scalar of the dtau matrices in the
// workspace; KM: scalar of the packed Minv in the workspace
// products == false: only the Minv output (symmetric, or upper with zeros below when minv_upper)
template <class S, class W, class KM>
int launch_minv_products(const gb_model* M, long B, const KM* wsMi, Arr Minv, const W* wsP,
                         const gb::DerivLayout& L, Arr o0, Arr o1, cudaStream_t st, bool products = true,
                         bool minv_upper = false) {
  if constexpr (std::is_same<S, float>::value && std::is_same<W, float>::value &&
                std::is_same<KM, gb::dfloat>::value) {
    if (products) {
      bool used = false;
      const int rc = launch_products_pipe(M, B, wsMi, Minv, minv_upper, wsP, L.nP, o0, o1, st, used);
      if (rc != GB_OK || used) return rc;
    }
  }
  const long nn = (long)M->nv * M->nv, npk = (long)M->nv * (M->nv + 1) / 2;
  const int ngroup = reinterpret_cast<const gb::BlobHeader*>(M->blob.data())->ngroup;
  const int nrel = reinterpret_cast<const gb::BlobHeader*>(M->blob.data())->n_grp_rel;
  auto smem_of = [&](long G, int NM) {
    const long region = std::max(npk * G * (long)sizeof(KM), (NM * nn + 8) * G * (long)sizeof(S));
    return nn * G * (long)sizeof(S) + ((region + 15) & ~15L) + (long)sizeof(int) * (4 * ngroup + nrel);
  };
#ifndef GB_MINV_SMEM_KB
#define GB_MINV_SMEM_KB 100
#endif
  const long budget = GB_MINV_SMEM_KB * 1024;  // shared memory per CTA (100 KB: two CTAs per SM)
  int NM = products ? 2 : 0, lgG = 3;
  while (lgG > 0 && smem_of(1L << lgG, NM) > budget) --lgG;
  if (products && smem_of(1L << lgG, NM) > budget) NM = 1;
  if (smem_of(1L << lgG, NM) > 220 * 1024) return set_error(GB_ERR_UNSUPPORTED, "nv too large for the Minv products");
  const long G = 1L << lgG;
  const size_t smem = (size_t)smem_of(G, NM);
  const void* kern = lgG == 3 ? (const void*)k_minv_products<3, S, W, KM>
                   : lgG == 2 ? (const void*)k_minv_products<2, S, W, KM>
                   : lgG == 1 ? (const void*)k_minv_products<1, S, W, KM>
                              : (const void*)k_minv_products<0, S, W, KM>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_error(e, "k_minv_products");
  const long nit = ((B + kBlk - 1) / kBlk) * (kBlk / G);
  const long grid = std::min<long>(nit, (long)M->sm_count * 2 * 8);
  for (int m0 = 0; m0 < 2; m0 += (NM > 0 ? NM : 2)) {
    const unsigned char* bl = M->d_blob;
    const long nP = L.nP, dtq = L.dtq, dtv = L.dtv;
    const bool up = minv_upper;
    if (lgG == 3) k_minv_products<3, S, W, KM><<<(unsigned)grid, 512, smem, st>>>(bl, B, m0, NM, wsMi, Minv, up, wsP, nP, dtq, dtv, o0, o1);
    else if (lgG == 2) k_minv_products<2, S, W, KM><<<(unsigned)grid, 512, smem, st>>>(bl, B, m0, NM, wsMi, Minv, up, wsP, nP, dtq, dtv, o0, o1);
    else if (lgG == 1) k_minv_products<1, S, W, KM><<<(unsigned)grid, 512, smem, st>>>(bl, B, m0, NM, wsMi, Minv, up, wsP, nP, dtq, dtv, o0, o1);
    else k_minv_products<0, S, W, KM><<<(unsigned)grid, 512, smem, st>>>(bl, B, m0, NM, wsMi, Minv, up, wsP, nP, dtq, dtv, o0, o1);
    const int rc = cuda_error(cudaGetLastError(), "k_minv_products");
    if (rc != GB_OK) return rc;
  }
  return GB_OK;
}

template <class S, bool FE = false>
int run_rnea_derivs(const gb_model* M, long B, bool symmetric, Arr q, Arr v, Arr a, Arr dq, Arr dv, Arr Mo, Arr tau,
                    cudaStream_t st, Arr fext = Arr{nullptr, 0, 0}) {
  const gb::DerivLayout L = gb::make_deriv_layout(M->nj, M->nv, M->nslot, false);
  Workspace ws;
  int rc = ws_alloc(ws, sizeof(S) * (size_t)L.nS * B, st);
  if (rc != GB_OK) return rc;
  rc = blob_smem(M, M->has_three ? (const void*)k_rnea_derivs<S, FE, true> : (const void*)k_rnea_derivs<S, FE, false>,
                 "k_rnea_derivs");
  if (rc != GB_OK) return rc;
  // instance-layout matrices of a large batch are written coalesced into an SOA scratch, then transposed
  const long nn = (long)M->nv * M->nv;
  const bool staged = dq.es == 1 && B >= kSoaStagingMin;
  Workspace soa;
  Arr mats[3] = {dq, dv, Mo};
  if (staged) {
    rc = ws_alloc(soa, sizeof(double) * 3 * (size_t)nn * B, st);
    if (rc != GB_OK) return rc;
    for (int k = 0; k < 3; ++k) mats[k] = Arr{static_cast<double*>(soa.p) + (size_t)k * nn * B, 1, B};
  }
  // the three matrices are cleared with full-bandwidth memsets; the kernel writes their non-zero entries
  for (const Arr& a : mats) {
    rc = cuda_error(cudaMemsetAsync(const_cast<double*>(a.p), 0, sizeof(double) * (size_t)nn * B, st), "cudaMemsetAsync");
    if (rc != GB_OK) return rc;
  }
  const int tpb = M->tpb[GB_FUNC_RNEA_DERIVATIVES];
  const long grid = (B + tpb - 1) / tpb;
  if (M->has_three)
    k_rnea_derivs<S, FE, true><<<(unsigned)grid, tpb, M->stage_bytes, st>>>(M->d_blob, M->stage_bytes, B, L,
                                                                       static_cast<S*>(ws.p), symmetric, q, v, a,
                                                                       mats[0], mats[1], mats[2], tau, fext);
  else
    k_rnea_derivs<S, FE, false><<<(unsigned)grid, tpb, M->stage_bytes, st>>>(M->d_blob, M->stage_bytes, B, L,
                                                                       static_cast<S*>(ws.p), symmetric, q, v, a,
                                                                       mats[0], mats[1], mats[2], tau, fext);
  rc = cuda_error(cudaGetLastError(), "k_rnea_derivs");
  if (rc != GB_OK || !staged) return rc;
  const Arr outs[3] = {dq, dv, Mo};
  for (int k = 0; k < 3; ++k) {
    rc = launch_soa_to_instance(mats[k].p, B, nn, outs[k], st);
    if (rc != GB_OK) return rc;
  }
  return GB_OK;
}

// The three sweep kernels of the ABA derivatives on a workspace laid out by
// aba_ws_layout, in the model's layout (gb_sweeps_t*.cu, one translation unit
// per team size).
// With external forces (fext.p set) the sweeps run one thread per configuration.
template <class S, class T3, class T, class K, class SS, class P>
int launch_aba_sweeps(const gb_model* M, long B, Arr q, Arr v, Arr tau, Arr ddq, void* ws, cudaStream_t st,
                      Arr fext = Arr{nullptr, 0, 0}) {
  constexpr bool f64 = std::is_same<K, double>::value, vjp = std::is_same<P, gb::dfloat>::value;
  constexpr bool df = std::is_same<S, gb::dfloat>::value;  // double-float column sets (deep trees)
  const SweepCall c{f64 ? kSweepFp64 : df ? kSweepMixedDf : vjp ? kSweepMixedVjp : kSweepMixed, M, B, q, v, tau, ddq,
                    ws, st, fext};
  return fext.p ? sweeps_t1(c) : sweeps_team(c);
}

template <class S, class T3, class T, class K, class SS, class P>
int launch_aba_derivs_ws(const gb_model* M, long B, Arr q, Arr v, Arr tau, Arr dq, Arr dv, Arr Minv, Arr ddq, void* ws,
                         cudaStream_t st, Arr fext = Arr{nullptr, 0, 0}) {
  int rc = launch_aba_sweeps<S, T3, T, K, SS, P>(M, B, q, v, tau, ddq, ws, st, fext);
  if (rc != GB_OK) return rc;
  const gb::DerivLayout L = gb::make_deriv_layout(M->nj, M->nv, M->nslot, true);
  const AbaWs W = aba_ws_layout<S, K, SS, P>(L, M->nv, B);
  char* base = static_cast<char*>(ws);
  return launch_minv_products<P, P, K>(M, B, reinterpret_cast<K*>(base + W.oMB), Minv,
                                       reinterpret_cast<P*>(base + W.oP), L, dq, dv, st);
}

// Vector-Jacobian products of the forward dynamics for an incoming gradient g on
// ddq: tau_bar = Minv g, q_bar = ddq_dq^T g = -dtau_dq^T (Minv g), v_bar =
// -dtau_dv^T (Minv g) (Minv symmetric) -- O(nv^2) per configuration from the
// workspace of the sweeps, instead of the O(nv^3) products.  A warp per
// configuration: lanes over rows of Minv g, then over columns of dtau.
template <class A, class W, class KM>
__global__ void __launch_bounds__(256)
    k_aba_vjp(const unsigned char* blob, long B, const KM* wsMB, const W* wsP, long nP, long dtq, long dtv, Arr g,
              Arr qb, Arr vb, Arr tb) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const gb::BlobHeader* h = reinterpret_cast<const gb::BlobHeader*>(blob);
  const int nv = h->nv, nrel = h->n_rel, npk = nv * (nv + 1) / 2;
  int* srel_off = reinterpret_cast<int*>(smem_raw);
  int* srel = srel_off + (nv + 1);
  A* sw = reinterpret_cast<A*>(smem_raw + (((size_t)(nv + 1 + nrel) * sizeof(int) + 15) & ~(size_t)15));
  for (int t = threadIdx.x; t <= nv; t += blockDim.x) srel_off[t] = reinterpret_cast<const int*>(blob + h->o_rel_off)[t];
  for (int t = threadIdx.x; t < nrel; t += blockDim.x) srel[t] = reinterpret_cast<const int*>(blob + h->o_rel_list)[t];
  __syncthreads();
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32, nwarps = blockDim.x / 32;
  A* gs = sw + (long)warp * 2 * nv;
  A* ys = gs + nv;
  for (long b = (long)blockIdx.x * nwarps + warp; b < B; b += (long)gridDim.x * nwarps) {
    for (int j = lane; j < nv; j += 32) gs[j] = A(g.p[b * g.is + (long)j * g.es]);
    __syncwarp();
    const KM* Mb = wsMB + (b / kBlk) * (long)npk * kBlk + (b % kBlk);
    for (int k = lane; k < nv; k += 32) {
      A acc = A(0);
      for (int j = 0; j < nv; ++j) acc += A(Mb[(long)(k <= j ? gb::upk(nv, k, j) : gb::upk(nv, j, k)) * kBlk]) * gs[j];
      ys[k] = acc;
      const_cast<double*>(tb.p)[b * tb.is + (long)k * tb.es] = to_double(acc);
    }
    __syncwarp();
    const W* Pb = wsP + (b / kBlk) * nP * kBlk + (b % kBlk);
    for (int c = lane; c < nv; c += 32) {
      A aq = A(0), av = A(0);
      for (int kk = srel_off[c]; kk < srel_off[c + 1]; ++kk) {
        const int k = srel[kk];
        const A y = ys[k];
        aq += A(Pb[(dtq + (long)k * nv + c) * kBlk]) * y;
        av += A(Pb[(dtv + (long)k * nv + c) * kBlk]) * y;
      }
      const_cast<double*>(qb.p)[b * qb.is + (long)c * qb.es] = -to_double(aq);
      const_cast<double*>(vb.p)[b * vb.is + (long)c * vb.es] = -to_double(av);
    }
    __syncwarp();
  }
}

// computeMinverse (reference algorithm/aba.hxx:838-880): passes 1-2 with zero
// velocity and torque (the bias terms vanish; Minv does not depend on them),
// the Minv recursion of pass 3, and the Minv output of the product kernel.
template <class K, class SS>
int run_minverse(const gb_model* M, long B, Arr q, Arr Minv, bool upper, cudaStream_t st) {
  const gb::DerivLayout L = gb::make_deriv_layout(M->nj, M->nv, M->nslot, true);
  const AbaWs W = aba_ws_layout<K, K, SS, K>(L, M->nv, B);
  Workspace ws;
  int rc = ws_alloc(ws, W.oP, st);  // no dtau region
  if (rc != GB_OK) return rc;
  K* wsMB = reinterpret_cast<K*>(static_cast<char*>(ws.p) + W.oMB);
  const gb::BlobHeader* h = reinterpret_cast<const gb::BlobHeader*>(M->blob.data());
  const Arr zero{reinterpret_cast<const double*>(M->d_blob + h->o_zero), 0, 0};
  const SweepCall c{std::is_same<K, double>::value ? kMinvFp64 : kMinvMixed, M, B, q, zero, zero, Arr{nullptr, 0, 0},
                    ws.p, st};
  rc = sweeps_team(c);
  if (rc != GB_OK) return rc;
  const Arr none{nullptr, 0, 0};
  return launch_minv_products<K, K, K>(M, B, wsMB, Minv, static_cast<const K*>(nullptr), L, none, none, st, false,
                                       upper);
}

template <class S, class T3, class T, class K, class SS, class P>
int run_aba_vjp(const gb_model* M, long B, Arr q, Arr v, Arr tau, Arr g, Arr qb, Arr vb, Arr tb, Arr ddq,
                cudaStream_t st) {
  const gb::DerivLayout L = gb::make_deriv_layout(M->nj, M->nv, M->nslot, true);
  const AbaWs W = aba_ws_layout<S, K, SS, P>(L, M->nv, B);
  Workspace ws;
  int rc = ws_alloc(ws, W.bytes, st);
  if (rc != GB_OK) return rc;
  rc = launch_aba_sweeps<S, T3, T, K, SS, P>(M, B, q, v, tau, ddq, ws.p, st);
  if (rc != GB_OK) return rc;
  const gb::BlobHeader* h = reinterpret_cast<const gb::BlobHeader*>(M->blob.data());
  constexpr int threads = 256;
  // accumulated in K (Minv is stored in K; dtau is rounded to P)
  const size_t smem = (((size_t)(M->nv + 1 + h->n_rel) * sizeof(int) + 15) & ~(size_t)15) +
                      (size_t)(threads / 32) * 2 * M->nv * sizeof(K);
  cudaError_t e = cudaFuncSetAttribute(k_aba_vjp<K, P, K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_error(e, "k_aba_vjp");
  const long grid = std::min<long>((B + 7) / 8, (long)M->sm_count * 8 * 4);
  char* base = static_cast<char*>(ws.p);
  k_aba_vjp<K, P, K><<<(unsigned)grid, threads, smem, st>>>(M->d_blob, B, reinterpret_cast<K*>(base + W.oMB),
                                                             reinterpret_cast<P*>(base + W.oP), L.nP, L.dtq, L.dtv, g,
                                                             qb, vb, tb);
  return cuda_error(cudaGetLastError(), "k_aba_vjp");
}

template <class S, class T3, class T, class K, class SS, class P>
int run_aba_derivs(const gb_model* M, long B, Arr q, Arr v, Arr tau, Arr dq, Arr dv, Arr Minv, Arr ddq,
                   cudaStream_t st, Arr fext = Arr{nullptr, 0, 0}) {
  const gb::DerivLayout L = gb::make_deriv_layout(M->nj, M->nv, M->nslot, true);
  Workspace ws;
  int rc = ws_alloc(ws, aba_ws_layout<S, K, SS, P>(L, M->nv, B).bytes, st);
  if (rc != GB_OK) return rc;
  return launch_aba_derivs_ws<S, T3, T, K, SS, P>(M, B, q, v, tau, dq, dv, Minv, ddq, ws.p, st, fext);
}

// The mixed derivative sweeps keep the column sets and dtau in double-float on trees deeper
// than this: the conditioning of their mass matrix grows with the depth and amplifies the
// FP32 rounding of the column sets past the 1e-5 bar (measured: the 100-link chain at 2.9e-4
// with FP32 column sets; the 32-dof humanoid, depth 9, at 9e-6).
constexpr int kMixedDfDepth = 32;
bool mixed_df(const gb_model* M) { return M->max_depth > kMixedDfDepth; }

}  // namespace

int check_gravity(const gb_model* M) {
  if (M->gravity[3] != 0.0 || M->gravity[4] != 0.0 || M->gravity[5] != 0.0)
    return set_error(GB_ERR_GRAVITY, "The gravity must be a pure force vector, no angular part");
  return GB_OK;
}

// Per-model launch preparation (at creation, on the model's device): the warp-task plan
// of the pipelined product kernel and its shared-memory size, when the two stages fit.
int prepare_model_launches(gb_model* M) {
  M->prod_plan_ok = false;
  const gb::BlobHeader* h = reinterpret_cast<const gb::BlobHeader*>(M->blob.data());
  const PipeSmem P = pipe_smem(M->nv, h->ngroup, h->n_grp_rel);
  if (P.bytes > (size_t)M->smem_optin) return GB_OK;
  ProdPlan plan;
  if (!make_prod_plan(M, GB_PROD_CWARPS, plan)) return GB_OK;
  const cudaError_t e =
      cudaFuncSetAttribute(k_minv_products_pipe, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P.bytes);
  if (e != cudaSuccess) return cuda_error(e, "k_minv_products_pipe");
  std::copy(plan.woff, plan.woff + kProdMaxWarps + 1, M->prod_woff);
  std::copy(plan.task, plan.task + kProdMaxTasks, M->prod_task);
  M->prod_plan_ok = true;
  return GB_OK;
}

int sweeps_team(const SweepCall& c) {
  switch (c.M->layout[GB_FUNC_ABA_DERIVATIVES]) {
    case GB_INSTANCE_PER_WARP: return sweeps_t32(c);
    case GB_INSTANCE_PER_8_LANES: return sweeps_t8(c);
    case GB_INSTANCE_PER_4_LANES: return sweeps_t4(c);
    default: return sweeps_t1(c);
  }
}

// The ABA-derivative kernels on a workspace the caller provides (no allocation):
// total bytes needed for a batch, and the launch itself.
size_t aba_derivs_workspace_bytes(const gb_model* M, int precision, long B) {
  const gb::DerivLayout L = gb::make_deriv_layout(M->nj, M->nv, M->nslot, true);
  if (precision == GB_FP64) return aba_ws_layout<double, double, double, double>(L, M->nv, B).bytes;
  if (mixed_df(M)) return aba_ws_layout<gb::dfloat, gb::dfloat, double, gb::dfloat>(L, M->nv, B).bytes;
  return aba_ws_layout<float, gb::dfloat, double, float>(L, M->nv, B).bytes;
}

int launch_aba_derivs_on_workspace(const gb_model* M, int precision, long B, Arr q, Arr v, Arr tau, Arr dq, Arr dv,
                                   Arr Minv, Arr ddq, void* ws, cudaStream_t st) {
  if (const int rc = check_gravity(M)) return rc;
  if (precision == GB_FP64)
    return launch_aba_derivs_ws<double, double, double, double, double, double>(M, B, q, v, tau, dq, dv, Minv, ddq,
                                                                                ws, st);
  if (mixed_df(M))
    return launch_aba_derivs_ws<gb::dfloat, gb::dfloat, gb::dfloat, gb::dfloat, double, gb::dfloat>(
        M, B, q, v, tau, dq, dv, Minv, ddq, ws, st);
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

int gb_pipeline_timeouts(unsigned int* count, int reset) {
  if (count == nullptr) return gbi::set_error(GB_ERR_INVALID_ARGUMENT, "count is NULL");
  GB_TRY(gbi::cuda_error(cudaDeviceSynchronize(), "gb_pipeline_timeouts"));
  GB_TRY(gbi::cuda_error(cudaMemcpyFromSymbol(count, gbi::g_pipe_timeouts, sizeof(unsigned int)), "gb_pipeline_timeouts"));
  if (reset) {
    const unsigned int zero = 0;
    GB_TRY(gbi::cuda_error(cudaMemcpyToSymbol(gbi::g_pipe_timeouts, &zero, sizeof(unsigned int)), "gb_pipeline_timeouts"));
  }
  return GB_OK;
}

int gb_pipeline_wait_selftest(unsigned int limit_us, void* stream) {
  if (limit_us == 0 || limit_us > 100000) return gbi::set_error(GB_ERR_INVALID_ARGUMENT, "limit_us must be in 1..100000");
  gbi::k_wait_selftest<<<1, 32, 0, (cudaStream_t)stream>>>(1000ull * limit_us);
  return gbi::cuda_error(cudaGetLastError(), "k_wait_selftest");
}

}  // extern "C"

namespace gbi {
int launch_rnea_derivs_fext(const gb_model* M, int precision, long B, Arr q, Arr v, Arr a, Arr fext, Arr dq, Arr dv,
                            Arr Mo, cudaStream_t st) {
  if (precision == GB_FP64)
    return run_rnea_derivs<double, true>(M, B, false, q, v, a, dq, dv, Mo, Arr{nullptr, 0, 0}, st, fext);
  return run_rnea_derivs<float, true>(M, B, false, q, v, a, dq, dv, Mo, Arr{nullptr, 0, 0}, st, fext);
}
namespace {

int rnea_derivs_entry(const gb_model* M, int precision, int matrix_mode, int layout, long B, const double* q,
                      const double* v, const double* a, const double* fext, double* dtau_dq, double* dtau_dv,
                      double* Mo, double* tau, void* stream) {
  GB_TRY(gbi::check_common(M, precision, layout, B));
  if (matrix_mode != GB_MATRIX_UPPER && matrix_mode != GB_MATRIX_SYMMETRIC)
    return gbi::set_error(GB_ERR_INVALID_ARGUMENT, "unknown matrix mode");
  GB_TRY(gbi::check_gravity(M));
  if (B == 0) return GB_OK;
  GB_TRY(gbi::check_ptr(q, "q")); GB_TRY(gbi::check_ptr(v, "v")); GB_TRY(gbi::check_ptr(a, "a"));
  GB_TRY(gbi::check_ptr(dtau_dq, "dtau_dq")); GB_TRY(gbi::check_ptr(dtau_dv, "dtau_dv")); GB_TRY(gbi::check_ptr(Mo, "M"));
  if (tau) GB_TRY(gbi::check_ptr(tau, "tau"));
  if (fext) GB_TRY(gbi::check_ptr(fext, "fext"));
  const long nn = (long)M->nv * M->nv;
  using gbi::arr;
  const gbi::Arr Aq = arr(q, layout, B, M->nq), Av = arr(v, layout, B, M->nv), Aa = arr(a, layout, B, M->nv);
  const gbi::Arr Adq = arr(dtau_dq, layout, B, nn), Adv = arr(dtau_dv, layout, B, nn), AM = arr(Mo, layout, B, nn);
  const gbi::Arr At = arr(tau, layout, B, M->nv);
  const bool sym = matrix_mode == GB_MATRIX_SYMMETRIC;
  cudaStream_t st = (cudaStream_t)stream;
  if (fext) {
    const gbi::Arr Af = arr(fext, layout, B, 6L * M->nj_user);
    if (precision == GB_FP64) return gbi::run_rnea_derivs<double, true>(M, B, sym, Aq, Av, Aa, Adq, Adv, AM, At, st, Af);
    return gbi::run_rnea_derivs<float, true>(M, B, sym, Aq, Av, Aa, Adq, Adv, AM, At, st, Af);
  }
  if (precision == GB_FP64) return gbi::run_rnea_derivs<double>(M, B, sym, Aq, Av, Aa, Adq, Adv, AM, At, st);
  return gbi::run_rnea_derivs<float>(M, B, sym, Aq, Av, Aa, Adq, Adv, AM, At, st);
}

int aba_derivs_entry(const gb_model* M, int precision, int layout, long B, const double* q, const double* v,
                     const double* tau, const double* fext, double* ddq_dq, double* ddq_dv, double* Minv, double* ddq,
                     void* stream) {
  GB_TRY(gbi::check_common(M, precision, layout, B));
  GB_TRY(gbi::check_gravity(M));
  if (B == 0) return GB_OK;
  GB_TRY(gbi::check_ptr(q, "q")); GB_TRY(gbi::check_ptr(v, "v")); GB_TRY(gbi::check_ptr(tau, "tau"));
  GB_TRY(gbi::check_ptr(ddq_dq, "ddq_dq")); GB_TRY(gbi::check_ptr(ddq_dv, "ddq_dv")); GB_TRY(gbi::check_ptr(Minv, "Minv"));
  if (ddq) GB_TRY(gbi::check_ptr(ddq, "ddq"));
  if (fext) GB_TRY(gbi::check_ptr(fext, "fext"));
  const long nn = (long)M->nv * M->nv;
  using gbi::arr;
  const gbi::Arr Aq = arr(q, layout, B, M->nq), Av = arr(v, layout, B, M->nv), At = arr(tau, layout, B, M->nv);
  const gbi::Arr Adq = arr(ddq_dq, layout, B, nn), Adv = arr(ddq_dv, layout, B, nn), AMi = arr(Minv, layout, B, nn);
  const gbi::Arr Add = arr(ddq, layout, B, M->nv);
  const gbi::Arr Af = fext ? arr(fext, layout, B, 6L * M->nj_user) : gbi::Arr{nullptr, 0, 0};
  cudaStream_t st = (cudaStream_t)stream;
  if (precision == GB_FP64)
    return gbi::run_aba_derivs<double, double, double, double, double, double>(M, B, Aq, Av, At, Adq, Adv, AMi, Add,
                                                                               st, Af);
  if (gbi::mixed_df(M))
    return gbi::run_aba_derivs<gb::dfloat, gb::dfloat, gb::dfloat, gb::dfloat, double, gb::dfloat>(
        M, B, Aq, Av, At, Adq, Adv, AMi, Add, st, Af);
  return gbi::run_aba_derivs<float, float, gb::dfloat, gb::dfloat, double, float>(M, B, Aq, Av, At, Adq, Adv, AMi,
                                                                                 Add, st, Af);
}
}  // namespace
}  // namespace gbi

extern "C" {

int gb_rnea_derivatives(const gb_model* M, int precision, int matrix_mode, int layout, long B, const double* q,
                        const double* v, const double* a, double* dtau_dq, double* dtau_dv, double* Mo, double* tau,
                        void* stream) {
  return gbi::rnea_derivs_entry(M, precision, matrix_mode, layout, B, q, v, a, nullptr, dtau_dq, dtau_dv, Mo, tau,
                                stream);
}

int gb_rnea_derivatives_fext(const gb_model* M, int precision, int matrix_mode, int layout, long B, const double* q,
                             const double* v, const double* a, const double* fext, double* dtau_dq, double* dtau_dv,
                             double* Mo, double* tau, void* stream) {
  if (!fext) return gbi::set_error(GB_ERR_INVALID_ARGUMENT, "fext is NULL");
  return gbi::rnea_derivs_entry(M, precision, matrix_mode, layout, B, q, v, a, fext, dtau_dq, dtau_dv, Mo, tau,
                                stream);
}

int gb_aba_derivatives(const gb_model* M, int precision, int layout, long B, const double* q, const double* v,
                       const double* tau, double* ddq_dq, double* ddq_dv, double* Minv, double* ddq, void* stream) {
  return gbi::aba_derivs_entry(M, precision, layout, B, q, v, tau, nullptr, ddq_dq, ddq_dv, Minv, ddq, stream);
}

int gb_aba_derivatives_fext(const gb_model* M, int precision, int layout, long B, const double* q, const double* v,
                            const double* tau, const double* fext, double* ddq_dq, double* ddq_dv, double* Minv,
                            double* ddq, void* stream) {
  if (!fext) return gbi::set_error(GB_ERR_INVALID_ARGUMENT, "fext is NULL");
  return gbi::aba_derivs_entry(M, precision, layout, B, q, v, tau, fext, ddq_dq, ddq_dv, Minv, ddq, stream);
}

int gb_compute_minverse(const gb_model* M, int precision, int matrix_mode, int layout, long B, const double* q,
                        double* Minv, void* stream) {
  GB_TRY(gbi::check_common(M, precision, layout, B));
  if (matrix_mode != GB_MATRIX_UPPER && matrix_mode != GB_MATRIX_SYMMETRIC)
    return gbi::set_error(GB_ERR_INVALID_ARGUMENT, "unknown matrix mode");
  if (B == 0) return GB_OK;
  GB_TRY(gbi::check_ptr(q, "q")); GB_TRY(gbi::check_ptr(Minv, "Minv"));
  const gbi::Arr Aq = gbi::arr(q, layout, B, M->nq), AMi = gbi::arr(Minv, layout, B, (long)M->nv * M->nv);
  const bool upper = matrix_mode == GB_MATRIX_UPPER;
  cudaStream_t st = (cudaStream_t)stream;
  if (precision == GB_FP64) return gbi::run_minverse<double, double>(M, B, Aq, AMi, upper, st);
  return gbi::run_minverse<gb::dfloat, double>(M, B, Aq, AMi, upper, st);
}

int gb_aba_derivatives_vjp(const gb_model* M, int precision, int layout, long B, const double* q, const double* v,
                           const double* tau, const double* g, double* q_bar, double* v_bar, double* tau_bar,
                           double* ddq, void* stream) {
  GB_TRY(gbi::check_common(M, precision, layout, B));
  GB_TRY(gbi::check_gravity(M));
  if (B == 0) return GB_OK;
  GB_TRY(gbi::check_ptr(q, "q")); GB_TRY(gbi::check_ptr(v, "v")); GB_TRY(gbi::check_ptr(tau, "tau"));
  GB_TRY(gbi::check_ptr(g, "g")); GB_TRY(gbi::check_ptr(q_bar, "q_bar")); GB_TRY(gbi::check_ptr(v_bar, "v_bar"));
  GB_TRY(gbi::check_ptr(tau_bar, "tau_bar"));
  if (ddq) GB_TRY(gbi::check_ptr(ddq, "ddq"));
  using gbi::arr;
  const gbi::Arr Aq = arr(q, layout, B, M->nq), Av = arr(v, layout, B, M->nv), At = arr(tau, layout, B, M->nv);
  const gbi::Arr Ag = arr(g, layout, B, M->nv), Aqb = arr(q_bar, layout, B, M->nv), Avb = arr(v_bar, layout, B, M->nv);
  const gbi::Arr Atb = arr(tau_bar, layout, B, M->nv), Add = arr(ddq, layout, B, M->nv);
  cudaStream_t st = (cudaStream_t)stream;
  if (precision == GB_FP64)
    return gbi::run_aba_vjp<double, double, double, double, double, double>(M, B, Aq, Av, At, Ag, Aqb, Avb, Atb, Add,
                                                                            st);
  // dtau kept in double-float: a projection g^T ddq_dq cancels more than the Jacobian entries do
  if (gbi::mixed_df(M))
    return gbi::run_aba_vjp<gb::dfloat, gb::dfloat, gb::dfloat, gb::dfloat, double, gb::dfloat>(
        M, B, Aq, Av, At, Ag, Aqb, Avb, Atb, Add, st);
  return gbi::run_aba_vjp<float, float, gb::dfloat, gb::dfloat, double, gb::dfloat>(M, B, Aq, Av, At, Ag, Aqb, Avb,
                                                                                   Atb, Add, st);
}

}  // extern "C"
