// Vector kernels of the TFQMR and GMRES drivers (solver.cu): a plain SpMV
// on the permuted CSR, linear combinations, and dot products against a
// block of vectors with a fixed-order two-stage reduction (results are
// reproducible run to run).
#include <cuda_runtime.h>

#include "kernels.cuh"

namespace pg {
namespace {

constexpr int kKryBlock = 256;
constexpr int kDotBlocks = 64;  // first-stage blocks per dot product

__global__ void k_spmv_plain(int n, const int32_t *__restrict__ rp,
                             const int32_t *__restrict__ ci,
                             const double *__restrict__ val,
                             const double *__restrict__ x,
                             double *__restrict__ y) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    double acc = 0.;
    for (int32_t k = rp[i]; k < rp[i + 1]; ++k) acc += val[k] * x[ci[k]];
    y[i] = acc;
  }
}

__global__ void k_lincomb(int n, double a, const double *x, double b,
                          const double *y, double *out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x)
    out[i] = a * x[i] + (b != 0. ? b * y[i] : 0.);
}

// partial[k][blockIdx.x] = sum over this block's rows of V[k][i] * w[i]
__global__ void __launch_bounds__(kKryBlock)
k_mdot(int n, const double *__restrict__ V, size_t ld,
       const double *__restrict__ w, double *__restrict__ partial) {
  __shared__ double red[kKryBlock];
  const int k = blockIdx.y;
  const double *v = V + (size_t)k * ld;
  double acc = 0.;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x)
    acc += v[i] * w[i];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int h = kKryBlock / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[(size_t)k * gridDim.x + blockIdx.x] = red[0];
}

// out[k] = sum of the partials of k in block order
__global__ void k_mdot_sum(int nb, const double *__restrict__ partial,
                           double *__restrict__ out) {
  __shared__ double red[kDotBlocks];
  const int k = blockIdx.x;
  red[threadIdx.x] = threadIdx.x < nb ? partial[(size_t)k * nb + threadIdx.x] : 0.;
  __syncthreads();
  for (int h = kDotBlocks / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[k] = red[0];
}

// w[i] -= sum_k h[k] V[k][i] (k in order)
__global__ void k_vsub(int n, int kn, const double *__restrict__ V, size_t ld,
                       const double *__restrict__ h, double *__restrict__ w) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    double acc = 0.;
    for (int k = 0; k < kn; ++k) acc += h[k] * V[(size_t)k * ld + i];
    w[i] -= acc;
  }
}

int grid(int n) {
  const int g = (n + kKryBlock - 1) / kKryBlock;
  return g < 1216 ? (g > 0 ? g : 1) : 1216;
}

}  // namespace

void launch_spmv_plain(const SolverDev &d, const double *val, const double *x,
                       double *y, cudaStream_t st) {
  k_spmv_plain<<<grid(d.n), kKryBlock, 0, st>>>(d.n, d.prp, d.pci, val, x, y);
  count_launches(1);
}

void launch_lincomb(int n, double a, const double *x, double b,
                    const double *y, double *out, cudaStream_t st) {
  k_lincomb<<<grid(n), kKryBlock, 0, st>>>(n, a, x, b, y, out);
  count_launches(1);
}

void launch_mdot(int n, int kn, const double *V, size_t ld, const double *w,
                 double *partial, double *out, cudaStream_t st) {
  const dim3 g(kDotBlocks, kn);
  k_mdot<<<g, kKryBlock, 0, st>>>(n, V, ld, w, partial);
  k_mdot_sum<<<kn, kDotBlocks, 0, st>>>(kDotBlocks, partial, out);
  count_launches(2);
}

void launch_vsub(int n, int kn, const double *V, size_t ld, const double *h,
                 double *w, cudaStream_t st) {
  k_vsub<<<grid(n), kKryBlock, 0, st>>>(n, kn, V, ld, h, w);
  count_launches(1);
}

}  // namespace pg
