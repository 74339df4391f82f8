// Coarse correction of the two-level additive Schwarz preconditioner.
//
// The one-level preconditioner (block-Jacobi ILU(0) over the subdomains)
// has no global coupling: the smooth, low-energy error modes of a
// high-contrast pressure system (a light bubble in a heavy liquid) are
// corrected only a subdomain width per iteration, and BiCGStab spends most
// of its iterations on a plateau resolving them.  The coarse space is the
// classical one of Nicolaides (1987): one indicator vector per subdomain,
// Z = [z_1 .. z_K] with z_s = 1 on the rows of subdomain s.  The two-level
// additive preconditioner (Toselli & Widlund, Domain Decomposition Methods,
// 2005, sec. 2.5) is
//     M^-1 r = B_ILU r + Z A_c^-1 Z^T r,      A_c = Z^T A Z (K x K).
// A_c is summed per subdomain from the permuted CSR in FP64 in a fixed
// order, and inverted once per factorisation by in-place Gauss-Jordan
// elimination without pivoting (A_c is definite for the pressure systems; a
// pivot that vanishes, as for a pure-Neumann system, removes its coarse
// unknown).  The elimination runs in FP32: it is K^3 multiply-adds, which
// the FP32 pipes do about 64x faster than the FP64 pipe, and an approximate
// coarse inverse leaves the preconditioner a fixed linear operator as long
// as it is applied in FP64, which it is.  An application is then the K
// subdomain sums of the input (fused into the streamed ILU(0) sweeps), one
// K x K matrix-vector product accumulated in FP64 and a constant added to
// every row of a subdomain.  All reductions run in a fixed order, so
// results are reproducible.
#include <type_traits>

#include "dd.cuh"
#include "kernels.cuh"

namespace pg {
namespace {

constexpr int kCoarseBlock = 128;

// deterministic block sum (fixed tree); every thread gets the total
__device__ double block_sum(double v, double *red) {
  red[threadIdx.x] = v;
  __syncthreads();
  for (int h = blockDim.x / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  const double t = red[0];
  __syncthreads();
  return t;
}

// A_c row of subdomain s: per-thread partial sums per coarse column slot
// (entries strided by thread), then each slot summed over the threads in
// thread order
__global__ void __launch_bounds__(kCoarseBlock)
k_coarse_assemble(int K, const int32_t *__restrict__ sub_ptr,
                  const int32_t *__restrict__ prp,
                  const double *__restrict__ val,
                  const int32_t *__restrict__ cptr,
                  const int32_t *__restrict__ cnb,
                  const uint8_t *__restrict__ cslot, float *__restrict__ ac) {
  extern __shared__ double part[];  // [kCoarseBlock][S]
  const int s = blockIdx.x;
  const int S = cptr[s + 1] - cptr[s];
  for (int j = 0; j < S; ++j) part[threadIdx.x * S + j] = 0.;
  const int32_t e0 = prp[sub_ptr[s]], e1 = prp[sub_ptr[s + 1]];
  for (int32_t k = e0 + threadIdx.x; k < e1; k += kCoarseBlock)
    part[threadIdx.x * S + cslot[k]] += val[k];
  __syncthreads();
  for (int j = threadIdx.x; j < S; j += kCoarseBlock) {
    double sum = 0.;
    for (int t = 0; t < kCoarseBlock; ++t) sum += part[t * S + j];
    ac[(size_t)s * K + cnb[cptr[s] + j]] = (float)sum;
  }
}

// pivot row / column 0 and the diagonal before elimination
__global__ void k_gj_init(int K, const float *__restrict__ ac,
                          float *__restrict__ rowb, float *__restrict__ colb,
                          float *__restrict__ dg0) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= K) return;
  rowb[i] = ac[i];
  colb[i] = ac[(size_t)i * K];
  dg0[i] = ac[(size_t)i * K + i];
}

// Gauss-Jordan step k on the K x K matrix in place, row i = blockIdx.y
// (the pivot row and column of this step are read from rowb/colb[k & 1];
// the ones of step k+1 are written to the other half as they are computed)
__global__ void __launch_bounds__(256)
k_gj_step(int K, int k, float *__restrict__ ac, float *__restrict__ rowb,
          float *__restrict__ colb, const float *__restrict__ dg0) {
  const int i = blockIdx.y;
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= K) return;
  const int b = k & 1;
  const float piv = rowb[b * K + k];
  const float ip = fabsf(piv) > 1e-5f * fabsf(dg0[k]) ? 1.f / piv : 0.f;
  const float a_ik = colb[b * K + i], a_kj = rowb[b * K + j];
  const size_t idx = (size_t)i * K + j;
  float v;
  if (i == k && j == k)
    v = ip;
  else if (i == k)
    v = a_kj * ip;
  else if (j == k)
    v = -a_ik * ip;
  else
    v = ac[idx] - a_ik * (a_kj * ip);
  ac[idx] = v;
  if (k + 1 < K) {
    const int nb = b ^ 1;
    if (i == k + 1) rowb[nb * K + j] = v;
    if (j == k + 1) colb[nb * K + i] = v;
  }
}

// Z^T in: one sum per subdomain
__global__ void __launch_bounds__(kCoarseBlock)
k_coarse_sum(const int32_t *__restrict__ sub_ptr, const double *__restrict__ in,
             double *__restrict__ csum, const KScalars *__restrict__ sc) {
  if (sc && sc->done) return;
  __shared__ double red[kCoarseBlock];
  const int s = blockIdx.x;
  double acc = 0.;
  for (int32_t i = sub_ptr[s] + threadIdx.x; i < sub_ptr[s + 1]; i += kCoarseBlock)
    acc += in[i];
  const double t = block_sum(acc, red);
  if (threadIdx.x == 0) csum[s] = t;
}

__global__ void __launch_bounds__(kCoarseBlock)
k_coarse_sum_dd(const int32_t *__restrict__ sub_ptr,
                const float2 *__restrict__ in, double *__restrict__ csum,
                const KScalars *__restrict__ sc) {
  if (sc && sc->done) return;
  __shared__ double red[kCoarseBlock];
  const int s = blockIdx.x;
  DdAcc acc = dd_acc(make_float2(0.f, 0.f));
  for (int32_t i = sub_ptr[s] + threadIdx.x; i < sub_ptr[s + 1]; i += kCoarseBlock)
    dd_acc_add(acc, in[i]);
  const double t = block_sum(dd_acc_to_double(acc), red);
  if (threadIdx.x == 0) csum[s] = t;
}

// y_s = (A_c^-1)_s . csum, then z += y_s on the rows of subdomain s
template <class VT>
__global__ void __launch_bounds__(kCoarseBlock)
k_coarse_correct(int K, const int32_t *__restrict__ sub_ptr,
                 const float *__restrict__ ainv,
                 const double *__restrict__ csum, VT *__restrict__ z,
                 const KScalars *__restrict__ sc) {
  if (sc && sc->done) return;
  __shared__ double red[kCoarseBlock];
  const int s = blockIdx.x;
  const float *row = ainv + (size_t)s * K;
  double acc = 0.;
  for (int j = threadIdx.x; j < K; j += kCoarseBlock)
    acc += (double)row[j] * csum[j];
  const double y = block_sum(acc, red);
  if constexpr (std::is_same<VT, double>::value) {
    for (int32_t i = sub_ptr[s] + threadIdx.x; i < sub_ptr[s + 1]; i += kCoarseBlock)
      z[i] += y;
  } else {
    const float2 yd = dd_from(y);
    for (int32_t i = sub_ptr[s] + threadIdx.x; i < sub_ptr[s + 1]; i += kCoarseBlock)
      z[i] = dd_add(z[i], yd);
  }
}

}  // namespace

void launch_coarse_setup(const CoarseDev &c, const double *pvals,
                         const int32_t *prp, cudaGraphExec_t *gj_graph,
                         cudaStream_t st) {
  const int K = c.K;
  cudaMemsetAsync(c.ac, 0, (size_t)K * K * sizeof(float), st);
  const size_t smem = (size_t)kCoarseBlock * c.max_cnb * sizeof(double);
  k_coarse_assemble<<<K, kCoarseBlock, smem, st>>>(K, c.sub_ptr, prp, pvals,
                                                   c.cptr, c.cnb, c.cslot, c.ac);
  k_gj_init<<<(K + 255) / 256, 256, 0, st>>>(K, c.ac, c.rowb, c.colb, c.dg0);
  count_launches(2);
  // the K elimination steps: captured once into a graph, replayed (run
  // directly when the capture is not possible)
  const dim3 grid((K + 255) / 256, K);
  auto steps = [&]() {
    for (int k = 0; k < K; ++k)
      k_gj_step<<<grid, 256, 0, st>>>(K, k, c.ac, c.rowb, c.colb, c.dg0);
  };
  if (gj_graph && !*gj_graph) {
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed) == cudaSuccess) {
      steps();
      if (cudaStreamEndCapture(st, &g) == cudaSuccess && g &&
          cudaGraphInstantiate(gj_graph, g, 0) != cudaSuccess)
        *gj_graph = nullptr;
      if (g) cudaGraphDestroy(g);
    }
    cudaGetLastError();  // a failed capture falls back to direct launches
  }
  if (gj_graph && *gj_graph)
    cudaGraphLaunch(*gj_graph, st);
  else
    steps();
  count_launches(K);
}

void launch_coarse_apply(const CoarseDev &c, const double *in, double *z,
                         bool have_sums, const KScalars *sc, cudaStream_t st) {
  if (!have_sums) {
    k_coarse_sum<<<c.K, kCoarseBlock, 0, st>>>(c.sub_ptr, in, c.csum, sc);
    count_launches(1);
  }
  k_coarse_correct<double><<<c.K, kCoarseBlock, 0, st>>>(c.K, c.sub_ptr, c.ac,
                                                         c.csum, z, sc);
  count_launches(1);
}

void launch_coarse_apply_dd(const CoarseDev &c, const float2 *in, float2 *z,
                            bool have_sums, const KScalars *sc,
                            cudaStream_t st) {
  if (!have_sums) {
    k_coarse_sum_dd<<<c.K, kCoarseBlock, 0, st>>>(c.sub_ptr, in, c.csum, sc);
    count_launches(1);
  }
  k_coarse_correct<float2><<<c.K, kCoarseBlock, 0, st>>>(c.K, c.sub_ptr, c.ac,
                                                         c.csum, z, sc);
  count_launches(1);
}

}  // namespace pg
