// The three sweep kernels of the ABA derivatives (passes 1-2, pass 3, pass 4)
// and the two of computeMinverse, in every configuration layout: one thread
// per configuration, or a team of 4, 8 or 32 lanes (gb_sweeps_t*.cu compile one
// team size each, so the variants build in parallel).  Also the helpers the
// other derivative kernels share (model staging, blocked workspace layout,
// workspace regions).
#pragma once

#include <type_traits>

#include "gb_derivs.cuh"
#include "gb_internal.h"

namespace gbi {

// One sweep launch: what to run (precision and variant), on which workspace.
// kSweepMixedDf: the mixed sweeps with the column sets, pass 3's arithmetic and dtau in
// double-float (deep trees, whose mass-matrix conditioning amplifies FP32 rounding)
enum SweepKind { kSweepFp64, kSweepMixed, kSweepMixedVjp, kSweepMixedDf, kMinvFp64, kMinvMixed };
struct SweepCall {
  SweepKind kind;
  const gb_model* M;
  long B;
  Arr q, v, tau, ddq;  // computeMinverse: v = tau = a zero vector
  void* ws;
  cudaStream_t st;
  Arr fext;  // external forces (njoints x 6 per configuration, joint frames) or p == nullptr
};
int sweeps_team(const SweepCall& c);  // dispatches on the model's layout
int sweeps_t1(const SweepCall& c);
int sweeps_t4(const SweepCall& c);
int sweeps_t8(const SweepCall& c);
int sweeps_t32(const SweepCall& c);

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
  gb::MView m = gb::make_view(smem);
  gb::attach_status(m, blob);
  return m;
}
__device__ __forceinline__ gb::In in_at(const Arr& a, long b) { return gb::In{a.p + b * a.is, a.es}; }
__device__ __forceinline__ gb::Out out_at(const Arr& a, long b) {
  return gb::Out{const_cast<double*>(a.p) + b * a.is, a.es};
}

// The ABA-derivative sweeps as three kernels (passes 1-2, pass 3, pass 4), so
// that each keeps fewer values live than one fused kernel would (register use
// bounds the number of resident warps).  The workspace carries everything
// between them.
// Blocked workspace layout of the arrays the product kernel reads (Minv,
// dtau_dq, dtau_dv): configurations in blocks of kBlk, element e of
// configuration b at ((b / kBlk) * n + e) * kBlk + b % kBlk for an array of n
// elements -- a warp of the sweep kernels still accesses whole 32-byte
// segments, and one block is contiguous for the product kernel.
constexpr int kBlk = 8;
template <class T> __device__ __forceinline__ gb::Ws<T> blocked(T* base, long n, long b) {
  return gb::Ws<T>{base + (b / kBlk) * n * kBlk + (b % kBlk), kBlk};
}

// A sweep kernel runs one configuration per thread (TS == 1) or per team of TS
// consecutive lanes (gb::LaneTeam: the lanes split the loops over matrix
// columns) -- the layouts for deep trees and small batches, where one thread
// per configuration leaves the SMs nearly empty.  The workspace is
// [element][configuration] in every layout: a warp's accesses to the
// per-joint entries of its configurations stay coalesced.
template <int TS> __device__ __forceinline__ long sweep_config() {
  return ((long)blockIdx.x * blockDim.x + threadIdx.x) / TS;
}
#define GB_SWEEP_CALL(fn, ...)                                          \
  do {                                                                  \
    if constexpr (TS == 1) fn(__VA_ARGS__);                           \
    else fn(__VA_ARGS__, gb::LaneTeam<TS>((int)(threadIdx.x & 31))); \
  } while (0)

// FE: with external forces (read from fext; otherwise fext is not touched)
// J3: with the three-dof steps of spherical / planar joints (one thread per configuration)
template <class K, class SS, int TS, bool FE = false, bool J3 = false>
__global__ void __launch_bounds__(kThreads, GB_DERIV_MINB)
    k_aba_derivs_pass12(const unsigned char* blob, int bytes, long B, gb::DerivLayout L, K* wsK, SS* wsSS, K* wsMB,
                        int npk, Arr q, Arr v, Arr tau, Arr fext) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_model(blob, bytes, smem);
  const long b = sweep_config<TS>();
  if (b >= B) return;
  const gb::In fe = in_at(fext, b);
  GB_SWEEP_CALL((gb::aba_derivs_pass12<K, SS, J3>), m, L, gb::Ws<K>{wsK + b, B},
                gb::Ws<SS>{wsSS + b, B}, blocked(wsMB, npk, b), in_at(q, b), in_at(v, b), in_at(tau, b),
                FE ? &fe : nullptr);
}

template <class S, class T, class K, int TS, bool FE = false, bool J3 = false>
__global__ void __launch_bounds__(kThreads, GB_DERIV_MINB)
    k_aba_derivs_pass3(const unsigned char* blob, int bytes, long B, gb::DerivLayout L, S* wsS, K* wsK, K* wsMB,
                       int npk, Arr v, Arr ddq, Arr fext) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_model(blob, bytes, smem);
  const long b = sweep_config<TS>();
  if (b >= B) return;
  const gb::Out dd = out_at(ddq, b);
  const gb::In fe = in_at(fext, b);
  GB_SWEEP_CALL((gb::aba_derivs_pass3<S, T, K, false, J3>), m, L, m.slot, gb::Ws<S>{wsS + b, B},
                gb::Ws<K>{wsK + b, B}, blocked(wsMB, npk, b), in_at(v, b), ddq.p ? &dd : nullptr,
                FE ? &fe : nullptr);
}

// the Minv recursion of computeMinverse (pass 3 without velocities and column sets)
template <class K, int TS, bool J3 = false>
__global__ void __launch_bounds__(kThreads, GB_DERIV_MINB)
    k_minverse_pass3(const unsigned char* blob, int bytes, long B, gb::DerivLayout L, K* wsK, K* wsMB, int npk) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_model(blob, bytes, smem);
  const long b = sweep_config<TS>();
  if (b >= B) return;
  const gb::Ws<K> zk = gb::Ws<K>{wsK + b, B};
  GB_SWEEP_CALL((gb::aba_derivs_pass3<K, K, K, true, J3>), m, L, m.slot, zk, zk, blocked(wsMB, npk, b),
                gb::In{nullptr, 0}, nullptr, nullptr);
}

template <class S, class T, class K, class P, int TS, bool J3 = false>
__global__ void __launch_bounds__(kThreads, GB_DERIV_MINB)
    k_aba_derivs_pass4(const unsigned char* blob, int bytes, long B, gb::DerivLayout L, S* wsS, K* wsK, P* wsP) {
  extern __shared__ __align__(16) unsigned char smem[];
  const gb::MView m = stage_model(blob, bytes, smem);
  const long b = sweep_config<TS>();
  if (b >= B) return;
  GB_SWEEP_CALL((gb::aba_derivs_pass4<S, T, K, P, J3>), m, L, gb::Ws<S>{wsS + b, B},
                gb::Ws<K>{wsK + b, B}, blocked(wsP, L.nP, b));
}

int blob_smem(const gb_model* M, const void* kernel, const char* name) {
  if (M->stage_bytes > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, M->stage_bytes);
    if (e != cudaSuccess) return cuda_error(e, name);
  }
  return GB_OK;
}

// Workspace of the ABA derivatives, regions 256-byte aligned: SS (articulated
// inertias and u: FP64), K (kinematics, Fcrb columns, U Dinv, Dinv u, velocity
// / acceleration), S (the derivative column sets stored between passes 3 and
// 4: computed in T3 by pass 3 and in T by pass 4) -- these three [element]
// [configuration] -- and, in the blocked layout the product kernel reads, MB
// (the packed upper Minv, scalar K) and P (dtau_dq, dtau_dv in the scalar of
// the -Minv*dtau products).  The mixed kernels use K = T = dfloat and
// S = T3 = P = float.
struct AbaWs {
  size_t oK, oS, oMB, oP, bytes;
};
template <class S, class K, class SS, class P>
AbaWs aba_ws_layout(const gb::DerivLayout& L, int nv, long B) {
  auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t Bp = (size_t)((B + kBlk - 1) / kBlk) * kBlk;
  AbaWs w;
  w.oK = up(sizeof(SS) * (size_t)L.nSS * B);
  w.oS = w.oK + up(sizeof(K) * (size_t)L.nK * B);
  w.oMB = w.oS + up(sizeof(S) * (size_t)L.nS * B);
  w.oP = w.oMB + up(sizeof(K) * (size_t)nv * (nv + 1) / 2 * Bp);
  w.bytes = w.oP + up(sizeof(P) * (size_t)L.nP * Bp);
  return w;
}

// the CTA size and grid of the sweep kernels: tpb configurations per CTA, or kThreads / TS with a team each
template <int TS> void sweep_grid(const gb_model* M, long B, int& tpb, long& grid) {
  tpb = TS > 1 ? kThreads : M->tpb[GB_FUNC_ABA_DERIVATIVES];
  const long per = tpb / TS;
  grid = (B + per - 1) / per;
}

template <class S, class T3, class T, class K, class SS, class P, int TS, bool FE, bool J3>
int launch_sweeps_as(const gb_model* M, long B, const gb::DerivLayout& L, Arr q, Arr v, Arr tau, Arr ddq, SS* wsSS,
                     K* wsK, S* wsS, K* wsMB, P* wsP, int npk, cudaStream_t st, Arr fext) {
  int tpb;
  long grid;
  sweep_grid<TS>(M, B, tpb, grid);
  int rc = blob_smem(M, (const void*)k_aba_derivs_pass12<K, SS, TS, FE, J3>, "k_aba_derivs_pass12");
  if (rc == GB_OK) rc = blob_smem(M, (const void*)k_aba_derivs_pass3<S, T3, K, TS, FE, J3>, "k_aba_derivs_pass3");
  if (rc == GB_OK) rc = blob_smem(M, (const void*)k_aba_derivs_pass4<S, T, K, P, TS, J3>, "k_aba_derivs_pass4");
  if (rc != GB_OK) return rc;
  k_aba_derivs_pass12<K, SS, TS, FE, J3><<<(unsigned)grid, tpb, M->stage_bytes, st>>>(
      M->d_blob, M->stage_bytes, B, L, wsK, wsSS, wsMB, npk, q, v, tau, fext);
  rc = cuda_error(cudaGetLastError(), "k_aba_derivs_pass12");
  if (rc != GB_OK) return rc;
  k_aba_derivs_pass3<S, T3, K, TS, FE, J3><<<(unsigned)grid, tpb, M->stage_bytes, st>>>(
      M->d_blob, M->stage_bytes, B, L, wsS, wsK, wsMB, npk, v, ddq, fext);
  rc = cuda_error(cudaGetLastError(), "k_aba_derivs_pass3");
  if (rc != GB_OK) return rc;
  k_aba_derivs_pass4<S, T, K, P, TS, J3><<<(unsigned)grid, tpb, M->stage_bytes, st>>>(M->d_blob, M->stage_bytes, B,
                                                                                           L, wsS, wsK, wsP);
  return cuda_error(cudaGetLastError(), "k_aba_derivs_pass4");
}

template <class K, class SS, int TS, bool J3>
int minverse_sweeps_as(const gb_model* M, long B, const gb::DerivLayout& L, Arr q, Arr zero, SS* wsSS, K* wsK,
                       K* wsMB, int npk, cudaStream_t st) {
  int tpb;
  long grid;
  sweep_grid<TS>(M, B, tpb, grid);
  int rc = blob_smem(M, (const void*)k_aba_derivs_pass12<K, SS, TS, false, J3>, "k_aba_derivs_pass12");
  if (rc == GB_OK) rc = blob_smem(M, (const void*)k_minverse_pass3<K, TS, J3>, "k_minverse_pass3");
  if (rc != GB_OK) return rc;
  k_aba_derivs_pass12<K, SS, TS, false, J3><<<(unsigned)grid, tpb, M->stage_bytes, st>>>(
      M->d_blob, M->stage_bytes, B, L, wsK, wsSS, wsMB, npk, q, zero, zero, Arr{nullptr, 0, 0});
  rc = cuda_error(cudaGetLastError(), "k_aba_derivs_pass12");
  if (rc != GB_OK) return rc;
  k_minverse_pass3<K, TS, J3><<<(unsigned)grid, tpb, M->stage_bytes, st>>>(M->d_blob, M->stage_bytes, B, L, wsK,
                                                                                wsMB, npk);
  return cuda_error(cudaGetLastError(), "k_minverse_pass3");
}

template <class S, class T3, class T, class K, class SS, class P, int TS, bool FE, bool J3>
int aba_sweeps_on(const SweepCall& c) {
  const gb_model* M = c.M;
  const gb::DerivLayout L = gb::make_deriv_layout(M->nj, M->nv, M->nslot, true);
  const AbaWs W = aba_ws_layout<S, K, SS, P>(L, M->nv, c.B);
  char* base = static_cast<char*>(c.ws);
  return launch_sweeps_as<S, T3, T, K, SS, P, TS, FE, J3>(
      M, c.B, L, c.q, c.v, c.tau, c.ddq, reinterpret_cast<SS*>(base), reinterpret_cast<K*>(base + W.oK),
      reinterpret_cast<S*>(base + W.oS), reinterpret_cast<K*>(base + W.oMB), reinterpret_cast<P*>(base + W.oP),
      M->nv * (M->nv + 1) / 2, c.st, c.fext);
}

template <class K, class SS, int TS, bool J3>
int minverse_sweeps_on(const SweepCall& c) {
  const gb_model* M = c.M;
  const gb::DerivLayout L = gb::make_deriv_layout(M->nj, M->nv, M->nslot, true);
  const AbaWs W = aba_ws_layout<K, K, SS, K>(L, M->nv, c.B);
  char* base = static_cast<char*>(c.ws);
  return minverse_sweeps_as<K, SS, TS, J3>(M, c.B, L, c.q, c.v, reinterpret_cast<SS*>(base),
                                           reinterpret_cast<K*>(base + W.oK), reinterpret_cast<K*>(base + W.oMB),
                                           M->nv * (M->nv + 1) / 2, c.st);
}

// the kernels of one team size (and with or without the three-dof steps) for every precision and variant
template <int TS, bool J3>
int sweeps_kinds(const SweepCall& c) {
  using gb::dfloat;
  if (c.fext.p) {  // external forces: one thread per configuration, ddq and the derivatives
    if constexpr (TS == 1) {
      if (c.kind == kSweepFp64) return aba_sweeps_on<double, double, double, double, double, double, 1, true, J3>(c);
      if (c.kind == kSweepMixed) return aba_sweeps_on<float, float, dfloat, dfloat, double, float, 1, true, J3>(c);
      if (c.kind == kSweepMixedDf)
        return aba_sweeps_on<dfloat, dfloat, dfloat, dfloat, double, dfloat, 1, true, J3>(c);
    }
    return set_error(GB_ERR_INVALID_ARGUMENT, "external forces: unsupported sweep variant");
  }
  switch (c.kind) {
    case kSweepFp64: return aba_sweeps_on<double, double, double, double, double, double, TS, false, J3>(c);
    case kSweepMixed: return aba_sweeps_on<float, float, dfloat, dfloat, double, float, TS, false, J3>(c);
    case kSweepMixedVjp: return aba_sweeps_on<float, float, dfloat, dfloat, double, dfloat, TS, false, J3>(c);
    case kSweepMixedDf: return aba_sweeps_on<dfloat, dfloat, dfloat, dfloat, double, dfloat, TS, false, J3>(c);
    case kMinvFp64: return minverse_sweeps_on<double, double, TS, J3>(c);
    case kMinvMixed: return minverse_sweeps_on<dfloat, double, TS, J3>(c);
  }
  return set_error(GB_ERR_INVALID_ARGUMENT, "unknown sweep kind");
}
// models with spherical / planar joints run one configuration per thread (the layout setting
// refuses the others) with the three-dof steps compiled in
template <int TS>
int sweeps_for(const SweepCall& c) {
  if constexpr (TS == 1)
    if (c.M->has_three) return sweeps_kinds<1, true>(c);
  return sweeps_kinds<TS, false>(c);
}

}  // namespace
}  // namespace gbi
