// swe_diagnostics.cu -- volume and energy integrals of the state on the device.
//
// The reference's ComputeIntegrals (src/SpaceDisc.cpp:76-104, commented out in
// the snapshot) sums over cells A (h, h (u^2 + v^2) / 2, h^2 / 2 + h b).  Here
// every wet cell contributes its cell-average state (the reference integrates
// the reconstruction of partially-wet cells with a 10-level TriangAverage for
// the two energy terms; their volume term is the same).  The sums are a
// deterministic two-pass reduction: fixed blocks over fixed cell ranges, then
// one block over the partial sums in order.
#include "swe_engine.cuh"

namespace swe {
namespace {

constexpr int kBlocks = 608;  // 4 per SM on 152 SMs
constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) k_integrals(DevMesh m, const double* W, const double* U, const double* V,
                                                        int c0, int n, const int* __restrict__ to, double* partial) {
  __shared__ double s[3][kThreads];
  double a0 = 0., a1 = 0., a2 = 0.;
  // cells visited in the caller's order (to: caller's row -> device cell), so
  // that the sums are the same in every device order
  for (int q = blockIdx.x * kThreads + threadIdx.x; q < n; q += kBlocks * kThreads) {
    const int i = to ? to[c0 + q] : c0 + q;
    const double b = m.bc[i];
    const double h = W[i] - b;
    if (is_wet(h)) {
      const double A = m.area[i];
      const double u = U[i], v = V[i];
      a0 += A * h;
      a1 += A * (0.5 * h * (u * u + v * v));
      a2 += A * (0.5 * h * h + h * b);
    }
  }
  s[0][threadIdx.x] = a0;
  s[1][threadIdx.x] = a1;
  s[2][threadIdx.x] = a2;
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int k = 0; k < 3; ++k) s[k][threadIdx.x] += s[k][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < 3) partial[blockIdx.x * 3 + threadIdx.x] = s[threadIdx.x][0];
}

__global__ void k_integrals_final(const double* partial, double* out) {
  if (threadIdx.x < 3) {
    double t = 0.;
    for (int b = 0; b < kBlocks; ++b) t += partial[b * 3 + threadIdx.x];
    out[threadIdx.x] = t;
  }
}

}  // namespace

cudaError_t Engine::integrals(int64_t c0, int64_t n, double* out_host) {
  if (!d_integrals_) {
    d_integrals_ = dalloc<double>(3 * kBlocks + 3);
    if (!d_integrals_) return cudaErrorMemoryAllocation;
  }
  k_integrals<<<kBlocks, kThreads, 0, stream_>>>(mesh_, state(0, 0), state(0, 1), state(0, 2), (int)c0, (int)n,
                                                 d_cell_to, d_integrals_);
  k_integrals_final<<<1, 32, 0, stream_>>>(d_integrals_, d_integrals_ + 3 * kBlocks);
  launches_ += 2;
  cudaError_t e = cudaMemcpyAsync(out_host, d_integrals_ + 3 * kBlocks, 3 * sizeof(double), cudaMemcpyDeviceToHost,
                                  stream_);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream_);
  return e;
}

}  // namespace swe
