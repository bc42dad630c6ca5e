// swe_fp64_peak.cu -- measures this GPU's FP64 FMA throughput, the second
// ceiling of the step beside HBM bandwidth (every value on the path is FP64).
#include <cuda_runtime.h>

#include "../../include/swe_fvm_gb300.h"

namespace {

// 8 independent FMA chains per thread, `iters` rounds each.
__global__ void k_dfma(double* out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-9 + k;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
  }
  double s = 0.;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  if (s == 12345.678) out[0] = s;  // keeps the chains alive
}

}  // namespace

extern "C" swe_status swe_measure_fp64_peak(double* tflops) {
  if (!tflops) return SWE_ERR_INVALID_ARGUMENT;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return SWE_ERR_OUT_OF_MEMORY;
  const int blocks = sms * 8, threads = 256, iters = 4096;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_dfma<<<blocks, threads>>>(out, 64, 0.999999, 1e-7);  // warm-up
  float best = 1e30f;
  for (int r = 0; r < 5; ++r) {
    cudaEventRecord(e0);
    k_dfma<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaError_t e = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess) return SWE_ERR_CUDA;
  const double flops = 2.0 * 8.0 * (double)iters * blocks * threads;
  *tflops = flops / (best * 1e-3) / 1e12;
  return SWE_OK;
}

// ---------------------------------------------------------------------------
// Self-test of the integer-pipe division and square root (swe_fp64.cuh)
// against the hardware instructions on n pseudo-random operand pairs.

#include "swe_fp64.cuh"
#include "swe_dual.cuh"
#include "swe_flux_adjoint.cuh"

namespace {

__device__ __forceinline__ unsigned long long splitmix(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// operand classes: random bits anywhere; exponents near 1; significands near
// 1 (tiny fraction) or near 2 (all ones); random bits with the full exponent range
__device__ double make_operand(unsigned long long r, unsigned long long r2) {
  const unsigned mode = (unsigned)(r2 & 7u);
  unsigned long long sign = (r2 >> 8) & 1ull;
  unsigned long long exp, man = r & ((1ull << 52) - 1ull);
  switch (mode) {
    case 0: return __longlong_as_double((long long)r);  // anything, specials included
    case 1: exp = 1023 - 40 + ((r2 >> 16) % 81); break;
    case 2: exp = 1023 - 40 + ((r2 >> 16) % 81); man &= 0xFFFull; break;                       // 1 + tiny
    case 3: exp = 1023 - 40 + ((r2 >> 16) % 81); man |= ((1ull << 52) - 1ull) ^ 0xFFFull; break;  // near 2
    case 4: exp = 1 + ((r2 >> 16) % 2046); break;                                               // full normal range
    case 5: exp = 1 + ((r2 >> 16) % 60); break;                                                 // near underflow
    case 6: exp = 2046 - ((r2 >> 16) % 60); break;                                              // near overflow
    default:
      if (((r2 >> 40) & 3u) == 0u) return __longlong_as_double((long long)(sign << 63));  // +-0
      exp = 1023 + ((r2 >> 16) % 5) - 2;
      man = (r2 >> 20) & ((1ull << 52) - 1ull);
      break;
  }
  return __longlong_as_double((long long)((sign << 63) | (exp << 52) | man));
}

__global__ void k_fp64_selftest(long long n, unsigned long long seed, unsigned long long* counts) {
  unsigned long long bad_div = 0, bad_sqrt = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const unsigned long long r0 = splitmix(seed ^ (4ull * i)), r1 = splitmix(seed ^ (4ull * i + 1));
    const unsigned long long r2 = splitmix(seed ^ (4ull * i + 2)), r3 = splitmix(seed ^ (4ull * i + 3));
    const double a = make_operand(r0, r1), b = make_operand(r2, r3);
    const double q_soft = swe::ddiv_rn(a, b), q_hw = __ddiv_rn(a, b);
    const bool nan_both = (q_soft != q_soft) && (q_hw != q_hw);
    if (!nan_both && __double_as_longlong(q_soft) != __double_as_longlong(q_hw)) ++bad_div;
    const double x = fabs(a);
    const double s_soft = swe::dsqrt_rn(x), s_hw = __dsqrt_rn(x);
    const bool nan_both2 = (s_soft != s_soft) && (s_hw != s_hw);
    if (!nan_both2 && __double_as_longlong(s_soft) != __double_as_longlong(s_hw)) ++bad_sqrt;
  }
  if (bad_div) atomicAdd(counts, bad_div);
  if (bad_sqrt) atomicAdd(counts + 1, bad_sqrt);
}

}  // namespace

extern "C" swe_status swe_selftest_fp64(int64_t n, uint64_t seed, int64_t* div_mismatches, int64_t* sqrt_mismatches) {
  if (n <= 0 || !div_mismatches || !sqrt_mismatches) return SWE_ERR_INVALID_ARGUMENT;
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, 2 * sizeof(unsigned long long)) != cudaSuccess) return SWE_ERR_OUT_OF_MEMORY;
  cudaMemset(d, 0, 2 * sizeof(unsigned long long));
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  k_fp64_selftest<<<sms * 8, 256>>>(n, seed, d);
  unsigned long long h[2] = {0, 0};
  cudaError_t e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return SWE_ERR_CUDA;
  *div_mismatches = (int64_t)h[0];
  *sqrt_mismatches = (int64_t)h[1];
  return SWE_OK;
}

// ---------------------------------------------------------------------------
// Self-test of the hand-written flux reverse against the forward-mode
// Jacobian (Dual<7>) on random interface states.
namespace {

__global__ void k_flux_adj_selftest(int flux, int ws, int n, unsigned long long seed, double* maxerr) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  auto U = [&](int k) {
    return (double)(splitmix(seed ^ (16ull * i + k)) >> 11) * (1.0 / 9007199254740992.0);
  };
  const double ang = 6.283185307179586 * U(0);
  swe::EdgeGeom g;
  g.nx = cos(ang);
  g.ny = sin(ang);
  g.tx = -g.ny;
  g.ty = g.nx;
  g.b = 0.3 * U(1) - 0.1;
  g.lmin = 0.01;
  const int dry = (int)(U(2) * 8.0);  // sometimes a dry side
  swe::SideState L{g.b + (dry == 0 ? 0. : 0.01 + 0.5 * U(3)), U(4) - 0.5, U(5) - 0.5};
  swe::SideState R{g.b + (dry == 1 ? 0. : 0.01 + 0.5 * U(6)), U(7) - 0.5, U(8) - 0.5};
  if (dry == 0) L.u = L.v = 0.;
  if (dry == 1) R.u = R.v = 0.;
  const double lF[3] = {U(9) - 0.5, U(10) - 0.5, U(11) - 0.5};
  double lL[3] = {0., 0., 0.}, lR[3] = {0., 0., 0.}, lb = 0.;
  swe::flux_reverse(flux, ws, g, L, R, lF, lL, lR, &lb);
  typedef swe::Dual<7> D;
  D F[3];
  swe::flux_t(flux, ws, g.nx, g.ny, g.tx, g.ty, D::var(g.b, 6), D::var(L.w, 0), D::var(L.u, 1), D::var(L.v, 2),
              D::var(R.w, 3), D::var(R.u, 4), D::var(R.v, 5), F);
  const double hand[7] = {lL[0], lL[1], lL[2], lR[0], lR[1], lR[2], lb};
  // normwise difference of the 7-component adjoint
  double num = 0., den = 0.;
  for (int k = 0; k < 7; ++k) {
    const double ref = lF[0] * F[0].d[k] + lF[1] * F[1].d[k] + lF[2] * F[2].d[k];
    num = fmax(num, fabs(hand[k] - ref));
    den = fmax(den, fabs(ref));
  }
  double err = den > 0. ? num / den : num;
  // the reverse's own wave speeds must equal the forward plugin's bit for bit
  {
    const double ul = L.u * g.nx + L.v * g.ny, hl = L.w - g.b;
    const double ur = R.u * g.nx + R.v * g.ny, hr = R.w - g.b;
    const swe::WsFwd f = swe::ws_forward(ws, ul, hl, ur, hr);
    double a0, a1;
    switch (ws) {
      case 0: swe::Rusanov::speeds(ul, hl, ur, hr, &a0, &a1); break;
      case 1: swe::Davis::speeds(ul, hl, ur, hr, &a0, &a1); break;
      default: swe::Einfeldt::speeds(ul, hl, ur, hr, &a0, &a1); break;
    }
    if (__double_as_longlong(a0) != __double_as_longlong(f.a0) ||
        __double_as_longlong(a1) != __double_as_longlong(f.a1))
      err = 1.;
  }
  // exact max via integer atomics on the (non-negative) double bit pattern
  atomicMax((unsigned long long*)maxerr, (unsigned long long)__double_as_longlong(err));
}

}  // namespace

extern "C" swe_status swe_selftest_flux_adjoint(int32_t flux, int32_t wavespeed, int64_t n, uint64_t seed,
                                                double* max_rel_err) {
  if (!max_rel_err || n <= 0 || n > (1 << 26) || flux < 0 || flux > 1 || wavespeed < 0 || wavespeed > 2)
    return SWE_ERR_INVALID_ARGUMENT;
  double* d = nullptr;
  if (cudaMalloc(&d, sizeof(double)) != cudaSuccess) return SWE_ERR_OUT_OF_MEMORY;
  cudaMemset(d, 0, sizeof(double));
  k_flux_adj_selftest<<<(int)((n + 255) / 256), 256>>>(flux, wavespeed, (int)n, seed, d);
  cudaError_t e = cudaMemcpy(max_rel_err, d, sizeof(double), cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e == cudaSuccess ? SWE_OK : SWE_ERR_CUDA;
}
