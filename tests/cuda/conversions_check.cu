// Test program: the integer FP32 <-> FP64 conversions of csrc/gb_spatial.cuh
// (widen, narrow) against the hardware conversions, over edge cases and a
// seeded sweep of bit patterns.  Prints "conversions_ok" and exits 0 when every
// value agrees (values the functions flush to zero by design are compared with
// the signed zero).
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../pinocchio_gb300/csrc/gb_spatial.cuh"

__global__ void k_convert(const unsigned* f32, const unsigned long long* f64, int n, double* wid, double* wid_hw,
                          float* nar, float* nar_hw) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float x = __uint_as_float(f32[i]);
  wid[i] = gb::widen(x);
  wid_hw[i] = (double)x;
  const double y = __longlong_as_double((long long)f64[i]);
  nar[i] = gb::narrow(y);
  nar_hw[i] = (float)y;
}

static uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

int main() {
  std::vector<unsigned> f32 = {0u, 0x80000000u, 0x7f800000u, 0xff800000u, 0x7fc00000u, 0x7f7fffffu, 0x00800000u,
                               0x3f800000u, 0xbf800000u, 0x00000001u, 0x007fffffu};
  std::vector<unsigned long long> f64 = {0ull, 0x8000000000000000ull, 0x7ff0000000000000ull, 0x7ff8000000000000ull,
                                         0x3ff0000000000000ull, 0x47efffffe0000000ull, 0x47efffffefffffffull,
                                         0x47effffff0000000ull, 0x3810000000000000ull, 0x380fffffffffffffull,
                                         0x3ff0000010000000ull, 0x3ff0000030000000ull, 0x3ff0000010000001ull,
                                         0x0000000000000001ull};
  uint64_t s = 12345;
  for (int k = 0; k < 200000; ++k) {
    const uint64_t r = splitmix(s);
    f32.push_back((unsigned)r);
    // doubles across the FP32 range, and exact ties of the rounding
    uint64_t d = r;
    const uint64_t ex = 897 + (r >> 52) % 254;
    d = (d & 0x800fffffffffffffull) | (ex << 52);
    if (k % 4 == 0) d = (d & ~0x1fffffffull) | 0x10000000ull;
    f64.push_back(d);
  }
  while (f64.size() < f32.size()) f64.push_back(0);
  while (f32.size() < f64.size()) f32.push_back(0);
  const int n = (int)f32.size();
  unsigned* d32; unsigned long long* d64; double *w, *wh; float *a, *ah;
  cudaMalloc(&d32, n * 4); cudaMalloc(&d64, n * 8); cudaMalloc(&w, n * 8); cudaMalloc(&wh, n * 8);
  cudaMalloc(&a, n * 4); cudaMalloc(&ah, n * 4);
  cudaMemcpy(d32, f32.data(), n * 4, cudaMemcpyHostToDevice);
  cudaMemcpy(d64, f64.data(), n * 8, cudaMemcpyHostToDevice);
  k_convert<<<(n + 255) / 256, 256>>>(d32, d64, n, w, wh, a, ah);
  if (cudaDeviceSynchronize() != cudaSuccess) { std::printf("cuda error\n"); return 2; }
  std::vector<double> W(n), WH(n); std::vector<float> A(n), AH(n);
  cudaMemcpy(W.data(), w, n * 8, cudaMemcpyDeviceToHost); cudaMemcpy(WH.data(), wh, n * 8, cudaMemcpyDeviceToHost);
  cudaMemcpy(A.data(), a, n * 4, cudaMemcpyDeviceToHost); cudaMemcpy(AH.data(), ah, n * 4, cudaMemcpyDeviceToHost);
  long bad = 0;
  for (int i = 0; i < n; ++i) {
    const unsigned ex32 = (f32[i] >> 23) & 0xffu;
    double expect = WH[i];
    if (ex32 == 0) expect = (f32[i] >> 31) ? -0.0 : 0.0;  // subnormal inputs flush by design
    uint64_t b1, b2; std::memcpy(&b1, &W[i], 8); std::memcpy(&b2, &expect, 8);
    const bool nan = WH[i] != WH[i];
    if (nan ? (W[i] == W[i]) : (b1 != b2)) { if (bad < 5) std::printf("widen %08x\n", f32[i]); ++bad; }
    float expf = AH[i];
    const unsigned long long ex64 = (f64[i] >> 52) & 0x7ffull;
    if (ex64 < 897ull) expf = (f64[i] >> 63) ? -0.0f : 0.0f;  // below the FP32 normal range by design
    unsigned c1, c2; std::memcpy(&c1, &A[i], 4); std::memcpy(&c2, &expf, 4);
    if ((AH[i] != AH[i]) ? (A[i] == A[i]) : (c1 != c2)) { if (bad < 5) std::printf("narrow %016llx\n", f64[i]); ++bad; }
  }
  std::printf("%ld mismatches of %d\n", bad, n);
  if (bad == 0) std::printf("conversions_ok\n");
  return bad == 0 ? 0 : 1;
}
