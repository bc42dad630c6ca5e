// swe_noalloc.cu -- an edge-flux pass that allocates no device memory.
//
// Some callers cannot call cudaMalloc: code that runs while a framework owns
// every byte of device memory through its own pool, real-time loops where an
// allocation (and the implicit synchronisation it may bring) is forbidden, or
// plugins loaded into a host process that only hands them device pointers.
// swe_edge_fluxes_noalloc serves them: the caller passes the inputs and the
// outputs, and the only scratch the pass needs (one partial minimum of the
// length-to-wavespeed ratio per thread block) lives in a file-scope
// `static __device__` array of fixed size that every GPU loading this library
// holds until the process exits.
#include <cuda_runtime.h>

#include "../../include/swe_fvm_gb300.h"
#include "swe_physics.cuh"

namespace {

constexpr int kThreads = 256;
// 512 KB of partial minima: one per block of 256 edges, so at most
// 65536 x 256 = 16,777,216 edges per call.
constexpr int kMaxBlocks = 65536;
constexpr long long kMaxEdges = (long long)kMaxBlocks * kThreads;

__device__ __align__(256) double g_block_min[kMaxBlocks];

constexpr double kInf = __builtin_huge_val();

// Pass 1: the flux of every edge and the block minimum of the ratio.
template <class FLUX>
__global__ void __launch_bounds__(kThreads) k_flux_noalloc(int n, const double* __restrict__ geom,
                                                           const double* __restrict__ left,
                                                           const double* __restrict__ right, double cor,
                                                           double* __restrict__ flux, double* scratch) {
  __shared__ double s_min[kThreads / 32];
  const int e = blockIdx.x * kThreads + threadIdx.x;
  double lw = kInf;
  if (e < n) {
    swe::EdgeGeom g;
    g.nx = geom[6 * e];
    g.ny = geom[6 * e + 1];
    g.tx = geom[6 * e + 2];
    g.ty = geom[6 * e + 3];
    g.b = geom[6 * e + 4];
    g.lmin = geom[6 * e + 5];
    swe::SideState L{left[3 * e], left[3 * e + 1], left[3 * e + 2]};
    swe::SideState R{right[3 * e], right[3 * e + 1], right[3 * e + 2]};
    double F[3];
    FLUX::eval(g, L, R, cor, &lw, F);
    flux[3 * e] = F[0];
    flux[3 * e + 1] = F[1];
    flux[3 * e + 2] = F[2];
  }
#pragma unroll
  for (int off = 16; off; off >>= 1) lw = swe::smin(lw, __shfl_xor_sync(0xffffffffu, lw, off));
  if ((threadIdx.x & 31) == 0) s_min[threadIdx.x >> 5] = lw;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = s_min[0];
    for (int w = 1; w < kThreads / 32; ++w) m = swe::smin(m, s_min[w]);
    scratch[blockIdx.x] = m;  // every block writes its slot: nothing to clear
  }
}

// Pass 2: one block folds the partial minima into min(1, ...) (the ratio is
// reset to 1 before every flux pass, src/SpaceDisc.cpp:56).
__global__ void __launch_bounds__(kThreads) k_min_noalloc(int nblocks, const double* scratch, double* ratio) {
  __shared__ double s_min[kThreads / 32];
  double m = kInf;
  for (int b = threadIdx.x; b < nblocks; b += kThreads) m = swe::smin(m, scratch[b]);
#pragma unroll
  for (int off = 16; off; off >>= 1) m = swe::smin(m, __shfl_xor_sync(0xffffffffu, m, off));
  if ((threadIdx.x & 31) == 0) s_min[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 1.0;
    for (int w = 0; w < kThreads / 32; ++w) r = swe::smin(r, s_min[w]);
    *ratio = r;
  }
}

// Device address of g_block_min in the calling thread's current context.  A
// module-scope array has one address per context (and a new one after
// cudaDeviceReset), so no address is cached: cudaGetSymbolAddress is a
// host-side lookup that issues no stream work.  On the first call in a
// context it also loads this library's device code into that context, which
// is why that first call must come before any stream capture.
cudaError_t scratch_address(double** out) {
  void* p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_block_min);
  if (e != cudaSuccess) return e;
  *out = (double*)p;
  return cudaSuccess;
}

template <class FLUX>
void launch(int n, const double* geom, const double* left, const double* right, double cor, double* flux,
            double* ratio, double* scratch, cudaStream_t s) {
  const int blocks = (n + kThreads - 1) / kThreads;
  k_flux_noalloc<FLUX><<<blocks, kThreads, 0, s>>>(n, geom, left, right, cor, flux, scratch);
  k_min_noalloc<<<1, kThreads, 0, s>>>(blocks, scratch, ratio);
}

}  // namespace

extern "C" swe_status swe_edge_fluxes_noalloc(int32_t flux, int32_t wavespeed, int64_t n_edges,
                                              const double* edge_geom, const double* left, const double* right,
                                              double cor, double* flux_out, double* ratio_out, void* stream) {
  if (flux < 0 || flux > 1 || wavespeed < 0 || wavespeed > 2) return SWE_ERR_INVALID_ARGUMENT;
  if (n_edges <= 0 || n_edges > kMaxEdges) return SWE_ERR_INVALID_ARGUMENT;
  if (!edge_geom || !left || !right || !flux_out || !ratio_out) return SWE_ERR_INVALID_ARGUMENT;
  // An error left pending by earlier work on this thread is reported as such
  // (and left pending) instead of being consumed and blamed on these launches.
  if (cudaPeekAtLastError() != cudaSuccess) return SWE_ERR_CUDA;
  double* scratch = nullptr;
  if (scratch_address(&scratch) != cudaSuccess) return SWE_ERR_CUDA;
  cudaStream_t s = (cudaStream_t)stream;
  const int n = (int)n_edges;
  switch (flux * 3 + wavespeed) {
    case 0: launch<swe::HLL<swe::Rusanov>>(n, edge_geom, left, right, cor, flux_out, ratio_out, scratch, s); break;
    case 1: launch<swe::HLL<swe::Davis>>(n, edge_geom, left, right, cor, flux_out, ratio_out, scratch, s); break;
    case 2: launch<swe::HLL<swe::Einfeldt>>(n, edge_geom, left, right, cor, flux_out, ratio_out, scratch, s); break;
    case 3: launch<swe::HLLC<swe::Rusanov>>(n, edge_geom, left, right, cor, flux_out, ratio_out, scratch, s); break;
    case 4: launch<swe::HLLC<swe::Davis>>(n, edge_geom, left, right, cor, flux_out, ratio_out, scratch, s); break;
    default: launch<swe::HLLC<swe::Einfeldt>>(n, edge_geom, left, right, cor, flux_out, ratio_out, scratch, s);
  }
  return cudaGetLastError() == cudaSuccess ? SWE_OK : SWE_ERR_CUDA;
}
