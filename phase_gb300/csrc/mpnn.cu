// Learned initial guess for the pressure solve: a small message-passing
// network on the matrix graph (Gilmer et al., "Neural message passing for
// quantum chemistry", ICML 2017) with hand-written forward, backward and
// Adam (Kingma & Ba, ICLR 2015) kernels.  No reference counterpart: Phase
// always starts BiCGStab from its previous solution.
//
// Per cell i, from the system A x = b of this step and the previous
// solution x_prev:
//   features f_i = [x_prev_i / s_x, b_i / s_b, r_i / s_b, log(|a_ii| / m_a)]
//                  with r = b - A x_prev, s_* root-mean-square scales
//   h0 = relu(W0 f + b0)                                   (4 -> 32)
//   for l = 1..3:  q_j   = P_l h_j + c_l
//                  m_i   = sum_{j in N(i)} e_ij relu(q_j),  e_ij = -a_ij/a_ii
//                  h_l   = relu(U_l [h_{l-1}; m] + d_l) + h_{l-1}
//   guess_i = x_prev_i + s_d (w_o . h3_i + b_o),  s_d = rms(r_i / a_ii)
// Loss: |A g - b|^2 / |A x_prev - b|^2 + |g - x*|^2 / |x_prev - x*|^2.
// Weights are rounded to BF16 for every use (an FP32 master copy is kept for
// Adam); all accumulation is FP32.  Activations are stored feature-major
// (feature k of cell i at k*N + i) so every kernel reads coalesced.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>

#include <cmath>
#include <cstring>
#include <new>
#include <random>
#include <vector>

#include "internal.h"
#include "kernels.cuh"

namespace {

constexpr int H = 32;      // hidden width
constexpr int F = 4;       // input features
constexpr int L = 3;       // message-passing layers
constexpr int kBlock = 256;

inline int grid_of(int64_t n) {
  int64_t g = (n + kBlock - 1) / kBlock;
  return (int)(g < 4864 ? (g > 0 ? g : 1) : 4864);
}

// ---- parameter layout (FP32 master, offsets in floats) ----
struct Layout {
  int w0, b0, P[L], c[L], U[L], d[L], wo, bo, total;
  Layout() {
    int o = 0;
    w0 = o; o += F * H;
    b0 = o; o += H;
    for (int l = 0; l < L; ++l) {
      P[l] = o; o += H * H;
      c[l] = o; o += H;
      U[l] = o; o += 2 * H * H;
      d[l] = o; o += H;
    }
    wo = o; o += H;
    bo = o; o += 1;
    total = o;
  }
};

// ---------------------------------------------------------------- kernels
__global__ void k_round_bf16(int n, const float *__restrict__ src,
                             float *__restrict__ dst) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x)
    dst[i] = __bfloat162float(__float2bfloat16(src[i]));
}

// per-block sums of four doubles (fixed order: warp butterfly, then warps in
// order) written to part[blockIdx.x * 4 + k]; k_finish_sums adds the blocks'
// partials in block order, so the scales are reproducible
__device__ void block_sums4(const double (&s)[4], double *__restrict__ part) {
  __shared__ double ws[4][kBlock / 32];
  for (int k = 0; k < 4; ++k) {
    double v = s[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) ws[k][threadIdx.x >> 5] = v;
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    double t = 0.;
    for (int w = 0; w < kBlock / 32; ++w) t += ws[threadIdx.x][w];
    part[blockIdx.x * 4 + threadIdx.x] = t;
  }
}

__global__ void k_finish_sums(int nblk, const double *__restrict__ part,
                              double *__restrict__ sums) {
  __shared__ double red[4][kBlock];
  for (int k = 0; k < 4; ++k) {
    double t = 0.;
    for (int b = threadIdx.x; b < nblk; b += kBlock) t += part[b * 4 + k];
    red[k][threadIdx.x] = t;
  }
  __syncthreads();
  for (int h = kBlock / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h)
      for (int k = 0; k < 4; ++k) red[k][threadIdx.x] += red[k][threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x < 4) sums[threadIdx.x] = red[threadIdx.x][0];
}

// log|d| for any finite double without FP64 log: frexp splits off the
// binary exponent, FP32 log of the mantissa in [0.5, 1); log(1e-300) for 0
__device__ __forceinline__ float log_abs(double d) {
  if (d == 0.) return -690.7755f;
  int ex;
  const double m = frexp(fabs(d), &ex);
  return logf((float)m) + (float)ex * 0.69314718f;
}

// r = b - A x, diag a_ii, edge weights e_ij = -a_ij / a_ii, and per-block
// sums of x^2, b^2, (r/a_ii)^2, log|a_ii| for the feature scales
__global__ void __launch_bounds__(kBlock)
k_prep(int n, const int32_t *__restrict__ rp, const int32_t *__restrict__ ci,
       const double *__restrict__ a, const double *__restrict__ b,
       const double *__restrict__ xp, float *__restrict__ r,
       float *__restrict__ diag, float *__restrict__ e,
       double *__restrict__ part) {
  double s[4] = {0., 0., 0., 0.};  // x^2, b^2, (r/a)^2, log|a|
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    double ax = 0., dii = 0.;
    for (int k = rp[i]; k < rp[i + 1]; ++k) {
      ax += a[k] * xp[ci[k]];
      if (ci[k] == i) dii = a[k];
    }
    const double ri = b[i] - ax;
    r[i] = (float)ri;
    diag[i] = (float)dii;
    // edge weights and r / a_ii are FP32 quantities: one FP32 reciprocal
    // instead of FP64 division and products (FP64 is a slow pipe here)
    const float inv = dii != 0. ? 1.f / (float)dii : 0.f;
    for (int k = rp[i]; k < rp[i + 1]; ++k)
      e[k] = ci[k] == i ? 0.f : -(float)a[k] * inv;
    s[0] += xp[i] * xp[i];
    s[1] += b[i] * b[i];
    const float q = (float)ri * inv;
    s[2] += (double)(q * q);
    s[3] += (double)log_abs(dii);
  }
  block_sums4(s, part);
}

__global__ void __launch_bounds__(kBlock)
k_features(int n, const double *__restrict__ b, const double *__restrict__ xp,
           const float *__restrict__ r, const float *__restrict__ diag,
           const double *__restrict__ sums, float *__restrict__ f) {
  __shared__ double sc[3];
  if (threadIdx.x == 0) {
    sc[0] = 1. / (sqrt(sums[0] / n) + 1e-300);
    sc[1] = 1. / (sqrt(sums[1] / n) + 1e-300);
    sc[2] = sums[3] / n;
  }
  __syncthreads();
  const double isx = sc[0], isb = sc[1];
  const float la = (float)sc[2];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    f[0 * n + i] = (float)(xp[i] * isx);
    f[1 * n + i] = (float)(b[i] * isb);
    f[2 * n + i] = (float)(r[i] * isb);
    f[3 * n + i] = log_abs((double)diag[i]) - la;
  }
}

// Forward dense layer: Y[h][i] = act(sum_k X[k][i] W[k][h] + bias[h])
// (+ X[h][i] when RESID: the residual connection h_l + relu(...)), K inputs
// from X1 (rows 0..KA-1) and X2 (the rest), W K x HO row-major.  Each thread
// loads its inputs eight at a time (all eight loads in flight), the weights
// come from shared memory as float4 over h; the products are accumulated in
// the same order as k_dense, so results are identical.  Z (optional): the
// pre-activations, for the backward pass.
template <int K, int KA, int HO, bool RELU, bool RESID>
__global__ void __launch_bounds__(kBlock, 2)
k_dense_fwd(int n, const float *__restrict__ X1, const float *__restrict__ X2,
            const float *__restrict__ W, const float *__restrict__ bias,
            float *__restrict__ Y, float *__restrict__ Z) {
  static_assert(HO % 4 == 0, "HO must be a multiple of 4");
  __shared__ float4 w4[K * HO / 4];
  __shared__ float bs[HO];
  float *w = reinterpret_cast<float *>(w4);
  for (int t = threadIdx.x; t < K * HO; t += blockDim.x) w[t] = W[t];
  for (int t = threadIdx.x; t < HO; t += blockDim.x) bs[t] = bias ? bias[t] : 0.f;
  __syncthreads();
  constexpr int KC = K < 8 ? K : 8;  // inputs loaded together
  static_assert(K % KC == 0, "K must be a multiple of the load chunk");
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    float acc[HO];
#pragma unroll
    for (int h = 0; h < HO; ++h) acc[h] = bs[h];
#pragma unroll 1
    for (int k0 = 0; k0 < K; k0 += KC) {
      float x[KC];
#pragma unroll
      for (int u = 0; u < KC; ++u) {
        const int k = k0 + u;
        x[u] = k < KA ? X1[(size_t)k * n + i] : X2[(size_t)(k - KA) * n + i];
      }
#pragma unroll
      for (int u = 0; u < KC; ++u) {
        const int k = k0 + u;
#pragma unroll
        for (int q = 0; q < HO / 4; ++q) {
          const float4 wv = w4[k * (HO / 4) + q];
          acc[4 * q + 0] = fmaf(x[u], wv.x, acc[4 * q + 0]);
          acc[4 * q + 1] = fmaf(x[u], wv.y, acc[4 * q + 1]);
          acc[4 * q + 2] = fmaf(x[u], wv.z, acc[4 * q + 2]);
          acc[4 * q + 3] = fmaf(x[u], wv.w, acc[4 * q + 3]);
        }
      }
    }
#pragma unroll
    for (int h = 0; h < HO; ++h) {
      if (Z) Z[(size_t)h * n + i] = acc[h];
      float v = RELU ? fmaxf(acc[h], 0.f) : acc[h];
      if (RESID) v = X1[(size_t)h * n + i] + v;
      Y[(size_t)h * n + i] = v;
    }
  }
}

// Y[h][i] (+)= act( sum_k X[k][i] W[k][h] + bias[h] ) for K inputs taken
// from up to two feature-major arrays (X1 rows 0..K1-1, X2 the rest).
// W is K x H row-major (or H x K when transposed, for input gradients).
template <int K, int HO, bool RELU, bool ACC, bool TRANS>
__global__ void __launch_bounds__(kBlock)
k_dense(int n, const float *__restrict__ X1, int K1,
        const float *__restrict__ X2, const float *__restrict__ W,
        const float *__restrict__ bias, float *__restrict__ Y,
        float *__restrict__ Z) {
  __shared__ float w[K * HO];
  __shared__ float bs[HO];
  for (int t = threadIdx.x; t < K * HO; t += blockDim.x) {
    const int k = t / HO, h = t % HO;
    w[t] = TRANS ? W[h * K + k] : W[k * HO + h];
  }
  for (int t = threadIdx.x; t < HO; t += blockDim.x) bs[t] = bias ? bias[t] : 0.f;
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    float acc[HO];
#pragma unroll
    for (int h = 0; h < HO; ++h) acc[h] = bs[h];
    for (int k = 0; k < K; ++k) {
      const float x = k < K1 ? X1[(size_t)k * n + i] : X2[(size_t)(k - K1) * n + i];
#pragma unroll
      for (int h = 0; h < HO; ++h) acc[h] = fmaf(x, w[k * HO + h], acc[h]);
    }
#pragma unroll
    for (int h = 0; h < HO; ++h) {
      if (Z) Z[(size_t)h * n + i] = acc[h];  // pre-activation
      const float v = RELU ? fmaxf(acc[h], 0.f) : acc[h];
      if (ACC) Y[(size_t)h * n + i] += v;
      else Y[(size_t)h * n + i] = v;
    }
  }
}

// m[h][i] = sum_j e_ij relu(q[h][j])  (forward message)
__global__ void k_message(int n, const int32_t *__restrict__ rp,
                          const int32_t *__restrict__ ci,
                          const float *__restrict__ e,
                          const float *__restrict__ q, float *__restrict__ m) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    float acc[H];
#pragma unroll
    for (int h = 0; h < H; ++h) acc[h] = 0.f;
    for (int k = rp[i]; k < rp[i + 1]; ++k) {
      const float w = e[k];
      if (w == 0.f) continue;
      const int j = ci[k];
#pragma unroll
      for (int h = 0; h < H; ++h) acc[h] = fmaf(w, fmaxf(q[(size_t)h * n + j], 0.f), acc[h]);
    }
#pragma unroll
    for (int h = 0; h < H; ++h) m[(size_t)h * n + i] = acc[h];
  }
}

// dq[h][j] = relu'(q[h][j]) sum_{i in N(j)} e_ij dm[h][i]  (uses the
// transposed entry index: entry k = (j, i) -> tr[k] = index of (i, j))
__global__ void k_message_bwd(int n, const int32_t *__restrict__ rp,
                              const int32_t *__restrict__ ci,
                              const int32_t *__restrict__ tr,
                              const float *__restrict__ e,
                              const float *__restrict__ q,
                              const float *__restrict__ dm,
                              float *__restrict__ dq) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n;
       j += gridDim.x * blockDim.x) {
    float acc[H];
#pragma unroll
    for (int h = 0; h < H; ++h) acc[h] = 0.f;
    for (int k = rp[j]; k < rp[j + 1]; ++k) {
      const int i = ci[k];
      if (i == j || tr[k] < 0) continue;
      const float w = e[tr[k]];
#pragma unroll
      for (int h = 0; h < H; ++h) acc[h] = fmaf(w, dm[(size_t)h * n + i], acc[h]);
    }
#pragma unroll
    for (int h = 0; h < H; ++h)
      dq[(size_t)h * n + j] = q[(size_t)h * n + j] > 0.f ? acc[h] : 0.f;
  }
}

// dz = dy * (z > 0)
__global__ void k_relu_bwd(int64_t n, const float *__restrict__ z,
                           const float *__restrict__ dy,
                           float *__restrict__ dz) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dz[i] = z[i] > 0.f ? dy[i] : 0.f;
}

// G[k][h] += sum_i X[k][i] D[h][i]; gb[h] += sum_i D[h][i]   (weight grads)
template <int K>
__global__ void __launch_bounds__(kBlock)
k_wgrad(int n, const float *__restrict__ X1, int K1,
        const float *__restrict__ X2, const float *__restrict__ D,
        float *__restrict__ G, float *__restrict__ gb) {
  constexpr int CH = 32;  // cells staged per round
  __shared__ float xs[K][CH];
  __shared__ float ds[H][CH + 1];
  float acc[(K * H + kBlock - 1) / kBlock];
  float accb = 0.f;
  constexpr int PER = (K * H + kBlock - 1) / kBlock;
#pragma unroll
  for (int p = 0; p < PER; ++p) acc[p] = 0.f;
  for (int base = blockIdx.x * CH; base < n; base += gridDim.x * CH) {
    for (int t = threadIdx.x; t < K * CH; t += blockDim.x) {
      const int k = t / CH, c = t % CH, i = base + c;
      xs[k][c] = i < n ? (k < K1 ? X1[(size_t)k * n + i] : X2[(size_t)(k - K1) * n + i]) : 0.f;
    }
    for (int t = threadIdx.x; t < H * CH; t += blockDim.x) {
      const int h = t / CH, c = t % CH, i = base + c;
      ds[h][c] = i < n ? D[(size_t)h * n + i] : 0.f;
    }
    __syncthreads();
#pragma unroll
    for (int p = 0; p < PER; ++p) {
      const int t = threadIdx.x + p * kBlock;
      if (t < K * H) {
        const int k = t / H, h = t % H;
        float s = 0.f;
#pragma unroll 8
        for (int c = 0; c < CH; ++c) s = fmaf(xs[k][c], ds[h][c], s);
        acc[p] += s;
      }
    }
    if (threadIdx.x < H) {
      float s = 0.f;
      for (int c = 0; c < CH; ++c) s += ds[threadIdx.x][c];
      accb += s;
    }
    __syncthreads();
  }
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int t = threadIdx.x + p * kBlock;
    if (t < K * H) atomicAdd(&G[t], acc[p]);
  }
  if (gb && threadIdx.x < H) atomicAdd(&gb[threadIdx.x], accb);
}

// output head: out_i = wo . h_i + bo; guess = x_prev + s_d out
__global__ void k_head(int n, const float *__restrict__ h3,
                       const float *__restrict__ w, const double *__restrict__ xp,
                       const double *__restrict__ sums, float *__restrict__ out,
                       double *__restrict__ g) {
  const double sd = sqrt(sums[2] / n);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    float o = w[H];
#pragma unroll
    for (int h = 0; h < H; ++h) o = fmaf(w[h], h3[(size_t)h * n + i], o);
    out[i] = o;
    g[i] = xp[i] + sd * (double)o;
  }
}

// ---- inference: one kernel per layer, dense products on tensor cores ----
// A CTA takes a tile of kTile = 64 cells.  Its 128 threads gather the
// message m = sum_j e_ij relu(q_j) (FP32 FMAs in row order, as k_message)
// and stage [h | m] in shared memory as a 64 x 64 row-major tile; each warp
// then multiplies its 16 rows by U (64 x 32) and, for the next layer, the
// new h by P (32 x 32) with mma.sync m16n8k8 TF32.  The weights are BF16
// values, exact in TF32; each activation is split into a TF32 high part
// and a TF32 low part (two MMAs), so the products carry FP32 accuracy and
// only the summation order differs from the training forward.  h' and the
// next relu(q) are written back feature-major with coalesced stores.
constexpr int kTile = 64;          // cells per CTA tile
constexpr int kTileThreads = 128;  // 4 warps, 16 cells each
constexpr int kAS = 2 * H + 4;     // smem row stride of the [h | m] tile
constexpr int kWS = H + 8;         // smem row stride of a weight matrix

__device__ __forceinline__ uint32_t tf32_of(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ void mma_tf32(float (&c)[4], const uint32_t (&a)[4],
                                         uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// acc[nt] (+)= rows r0..r0+15 of the tile (columns c0..c0+K-1) times W
// (K x H in smem, stride kWS), for the warp's four 8-column n-tiles.
// Fragments of m16n8k8: a = A[g][t], A[g+8][t], A[g][t+4], A[g+8][t+4];
// b = B[t][g], B[t+4][g]; c = C[g][2t], C[g][2t+1], C[g+8][2t], C[g+8][2t+1]
// with g = lane / 4, t = lane % 4.
template <int K>
__device__ __forceinline__ void warp_gemm(float (&acc)[H / 8][4],
                                          const float *__restrict__ tile,
                                          int r0, int c0,
                                          const float *__restrict__ W) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int k0 = 0; k0 < K; k0 += 8) {
    const float av[4] = {tile[(r0 + g) * kAS + c0 + k0 + t],
                         tile[(r0 + g + 8) * kAS + c0 + k0 + t],
                         tile[(r0 + g) * kAS + c0 + k0 + t + 4],
                         tile[(r0 + g + 8) * kAS + c0 + k0 + t + 4]};
    uint32_t hi[4], lo[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      hi[q] = tf32_of(av[q]);
      lo[q] = tf32_of(av[q] - __uint_as_float(hi[q]));
    }
#pragma unroll
    for (int nt = 0; nt < H / 8; ++nt) {
      const uint32_t b0 = __float_as_uint(W[(k0 + t) * kWS + nt * 8 + g]);
      const uint32_t b1 = __float_as_uint(W[(k0 + t + 4) * kWS + nt * 8 + g]);
      mma_tf32(acc[nt], lo, b0, b1);
      mma_tf32(acc[nt], hi, b0, b1);
    }
  }
}

__device__ __forceinline__ void load_weights(float *__restrict__ dst,
                                             const float *__restrict__ W, int K) {
  for (int x = threadIdx.x; x < K * H; x += blockDim.x)
    dst[(x / H) * kWS + (x % H)] = W[x];
}

// features, h0 = relu(W0 f + b0) (FP32 FMAs) and relu(q_0) = relu(P_0 h0 +
// c_0) (tensor cores)
__global__ void __launch_bounds__(kTileThreads)
k_infer_in(int n, const double *__restrict__ b, const double *__restrict__ xp,
           const float *__restrict__ r, const float *__restrict__ diag,
           const double *__restrict__ sums, const float *__restrict__ W0,
           const float *__restrict__ b0, const float *__restrict__ P,
           const float *__restrict__ c, float *__restrict__ h0,
           float *__restrict__ q0) {
  __shared__ float tile[kTile * kAS];
  __shared__ float ps[H * kWS];
  __shared__ float w0s[F * H], bs0[H], cs[H];
  __shared__ double sc[3];
  load_weights(ps, P, H);
  for (int x = threadIdx.x; x < F * H; x += blockDim.x) w0s[x] = W0[x];
  for (int x = threadIdx.x; x < H; x += blockDim.x) {
    bs0[x] = b0[x];
    cs[x] = c[x];
  }
  if (threadIdx.x == 0) {
    sc[0] = 1. / (sqrt(sums[0] / n) + 1e-300);
    sc[1] = 1. / (sqrt(sums[1] / n) + 1e-300);
    sc[2] = sums[3] / n;
  }
  __syncthreads();
  const double isx = sc[0], isb = sc[1];
  const float la = (float)sc[2];
  const int cell = threadIdx.x & (kTile - 1), half = threadIdx.x / kTile;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int g = lane >> 2, t = lane & 3;
  const int n_tiles = (n + kTile - 1) / kTile;
  for (int tl = blockIdx.x; tl < n_tiles; tl += gridDim.x) {
    const int i = tl * kTile + cell;
    float hv[H / 2];
    if (i < n) {
      const float f[F] = {(float)(xp[i] * isx), (float)(b[i] * isb),
                          (float)(r[i] * isb), log_abs((double)diag[i]) - la};
#pragma unroll
      for (int k = 0; k < H / 2; ++k) {
        const int hh = half * (H / 2) + k;
        float a = bs0[hh];
#pragma unroll
        for (int u = 0; u < F; ++u) a = fmaf(f[u], w0s[u * H + hh], a);
        hv[k] = fmaxf(a, 0.f);
        h0[(size_t)hh * n + i] = hv[k];
      }
    } else {
#pragma unroll
      for (int k = 0; k < H / 2; ++k) hv[k] = 0.f;
    }
#pragma unroll
    for (int k = 0; k < H / 2; ++k) tile[cell * kAS + half * (H / 2) + k] = hv[k];
    __syncthreads();
    float acc[H / 8][4];
#pragma unroll
    for (int nt = 0; nt < H / 8; ++nt) {
      acc[nt][0] = acc[nt][2] = cs[nt * 8 + 2 * t];
      acc[nt][1] = acc[nt][3] = cs[nt * 8 + 2 * t + 1];
    }
    const int r0 = warp * 16;
    warp_gemm<H>(acc, tile, r0, 0, ps);
#pragma unroll
    for (int nt = 0; nt < H / 8; ++nt) {
      const int col = H + nt * 8 + 2 * t;
      tile[(r0 + g) * kAS + col] = fmaxf(acc[nt][0], 0.f);
      tile[(r0 + g) * kAS + col + 1] = fmaxf(acc[nt][1], 0.f);
      tile[(r0 + g + 8) * kAS + col] = fmaxf(acc[nt][2], 0.f);
      tile[(r0 + g + 8) * kAS + col + 1] = fmaxf(acc[nt][3], 0.f);
    }
    __syncthreads();
    if (i < n)
#pragma unroll
      for (int k = 0; k < H / 2; ++k) {
        const int hh = half * (H / 2) + k;
        q0[(size_t)hh * n + i] = tile[cell * kAS + H + hh];
      }
    __syncthreads();
  }
}

// one message-passing layer: m = sum_j e_ij relu(q_j),
// h' = h + relu(U [h; m] + d), then relu(q') = relu(P' h' + c') for the
// next layer, or (LAST) the head out = wo . h' + bo, g = x_prev + s_d out
template <bool LAST>
__global__ void __launch_bounds__(kTileThreads)
k_infer_layer(int n, const int32_t *__restrict__ rp,
              const int32_t *__restrict__ ci, const float *__restrict__ e,
              const float *__restrict__ qr, const float *__restrict__ hin,
              const float *__restrict__ U, const float *__restrict__ d,
              const float *__restrict__ P, const float *__restrict__ c,
              const float *__restrict__ wo, const double *__restrict__ xp,
              const double *__restrict__ sums, float *__restrict__ hout,
              float *__restrict__ qout, float *__restrict__ out,
              double *__restrict__ g) {
  __shared__ float tile[kTile * kAS];
  __shared__ float us[2 * H * kWS];
  __shared__ float ps[LAST ? 1 : H * kWS];
  __shared__ float ds[H], cs[H], wos[H + 1];
  load_weights(us, U, 2 * H);
  if (!LAST) load_weights(ps, P, H);
  for (int x = threadIdx.x; x < H; x += blockDim.x) {
    ds[x] = d[x];
    if (!LAST) cs[x] = c[x];
  }
  if (LAST)
    for (int x = threadIdx.x; x <= H; x += blockDim.x) wos[x] = wo[x];
  __syncthreads();
  const double sd = LAST ? sqrt(sums[2] / n) : 0.;
  const int cell = threadIdx.x & (kTile - 1), half = threadIdx.x / kTile;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int gq = lane >> 2, t = lane & 3;
  const int r0 = warp * 16;
  const int n_tiles = (n + kTile - 1) / kTile;
  for (int tl = blockIdx.x; tl < n_tiles; tl += gridDim.x) {
    const int i = tl * kTile + cell;
    // [h | m] of the tile, each thread half of one cell's features
    float m[H / 2], hv[H / 2];
#pragma unroll
    for (int k = 0; k < H / 2; ++k) m[k] = hv[k] = 0.f;
    if (i < n) {
#pragma unroll
      for (int k = 0; k < H / 2; ++k)
        hv[k] = hin[(size_t)(half * (H / 2) + k) * n + i];
      // edges four at a time: every gather of the four is issued before the
      // FMAs, which run in row order skipping zero weights (as k_message)
      const int k1 = rp[i + 1];
      for (int kb = rp[i]; kb < k1; kb += 4) {
        float w[4];
        int j[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const bool in = kb + u < k1;
          w[u] = in ? e[kb + u] : 0.f;
          j[u] = in ? ci[kb + u] : i;
        }
        float qv[4][H / 2];
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
          for (int k2 = 0; k2 < H / 2; ++k2)
            qv[u][k2] = qr[(size_t)(half * (H / 2) + k2) * n + j[u]];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          if (w[u] == 0.f) continue;
#pragma unroll
          for (int k2 = 0; k2 < H / 2; ++k2) m[k2] = fmaf(w[u], qv[u][k2], m[k2]);
        }
      }
    }
#pragma unroll
    for (int k = 0; k < H / 2; ++k) {
      tile[cell * kAS + half * (H / 2) + k] = hv[k];
      tile[cell * kAS + H + half * (H / 2) + k] = m[k];
    }
    __syncthreads();
    float acc[H / 8][4];
#pragma unroll
    for (int nt = 0; nt < H / 8; ++nt) {
      acc[nt][0] = acc[nt][2] = ds[nt * 8 + 2 * t];
      acc[nt][1] = acc[nt][3] = ds[nt * 8 + 2 * t + 1];
    }
    warp_gemm<2 * H>(acc, tile, r0, 0, us);
    __syncwarp();
    // h' = h + relu(acc) over the warp's own rows (columns 0..H-1)
#pragma unroll
    for (int nt = 0; nt < H / 8; ++nt) {
      const int col = nt * 8 + 2 * t;
      float *p0 = tile + (r0 + gq) * kAS + col, *p1 = tile + (r0 + gq + 8) * kAS + col;
      p0[0] = p0[0] + fmaxf(acc[nt][0], 0.f);
      p0[1] = p0[1] + fmaxf(acc[nt][1], 0.f);
      p1[0] = p1[0] + fmaxf(acc[nt][2], 0.f);
      p1[1] = p1[1] + fmaxf(acc[nt][3], 0.f);
    }
    __syncwarp();
    if (!LAST) {
#pragma unroll
      for (int nt = 0; nt < H / 8; ++nt) {
        acc[nt][0] = acc[nt][2] = cs[nt * 8 + 2 * t];
        acc[nt][1] = acc[nt][3] = cs[nt * 8 + 2 * t + 1];
      }
      warp_gemm<H>(acc, tile, r0, 0, ps);
      __syncwarp();
#pragma unroll
      for (int nt = 0; nt < H / 8; ++nt) {
        const int col = H + nt * 8 + 2 * t;
        tile[(r0 + gq) * kAS + col] = fmaxf(acc[nt][0], 0.f);
        tile[(r0 + gq) * kAS + col + 1] = fmaxf(acc[nt][1], 0.f);
        tile[(r0 + gq + 8) * kAS + col] = fmaxf(acc[nt][2], 0.f);
        tile[(r0 + gq + 8) * kAS + col + 1] = fmaxf(acc[nt][3], 0.f);
      }
    }
    __syncthreads();
    if (i < n) {
      if (LAST) {
        if (half == 0) {
          float o = wos[H];
#pragma unroll
          for (int k = 0; k < H; ++k) o = fmaf(wos[k], tile[cell * kAS + k], o);
          out[i] = o;
          g[i] = xp[i] + sd * (double)o;
        }
      } else {
#pragma unroll
        for (int k = 0; k < H / 2; ++k) {
          const int hh = half * (H / 2) + k;
          hout[(size_t)hh * n + i] = tile[cell * kAS + hh];
          qout[(size_t)hh * n + i] = tile[cell * kAS + H + hh];
        }
      }
    }
    __syncthreads();
  }
}

// residual res = A g - b, error err = g - x*, and per-block loss sums
// (k_finish_sums adds them into sums[4..7])
__global__ void __launch_bounds__(kBlock) k_loss(int n, const int32_t *__restrict__ rp,
                       const int32_t *__restrict__ ci,
                       const double *__restrict__ a,
                       const double *__restrict__ b,
                       const double *__restrict__ g,
                       const double *__restrict__ xs,
                       const double *__restrict__ xp, double *__restrict__ res,
                       double *__restrict__ err, double *__restrict__ part) {
  double s[4] = {0., 0., 0., 0.};  // |res|^2, |A xp - b|^2, |err|^2, |xp-x*|^2
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    double ag = 0., ap = 0.;
    for (int k = rp[i]; k < rp[i + 1]; ++k) {
      ag += a[k] * g[ci[k]];
      if (res) ap += a[k] * xp[ci[k]];
    }
    const double rr = ag - b[i];
    s[0] += rr * rr;
    if (res) {  // training: the residual vector and |A x_prev - b|^2 too
      const double r0 = ap - b[i];
      res[i] = rr;
      s[1] += r0 * r0;
    }
    if (xs) {
      const double ee = g[i] - xs[i], e0 = xp[i] - xs[i];
      err[i] = ee;
      s[2] += ee * ee;
      s[3] += e0 * e0;
    }
  }
  block_sums4(s, part);
}

// d out_i = s_d (2 (A^T res)_i / R0 + 2 err_i / E0)
__global__ void k_dout(int n, const int32_t *__restrict__ rp,
                       const int32_t *__restrict__ ci,
                       const int32_t *__restrict__ tr,
                       const double *__restrict__ a,
                       const double *__restrict__ res,
                       const double *__restrict__ err,
                       const double *__restrict__ sums,
                       float *__restrict__ dout) {
  const double sd = sqrt(sums[2] / n);
  const double R0 = sums[5] > 0. ? sums[5] : 1., E0 = sums[7] > 0. ? sums[7] : 1.;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    double atr = 0.;
    for (int k = rp[i]; k < rp[i + 1]; ++k)
      atr += a[tr[k] >= 0 ? tr[k] : k] * res[ci[k]];
    double d = 2. * atr / R0;
    if (err) d += 2. * err[i] / E0;
    dout[i] = (float)(sd * d);
  }
}

// head backward: dh3[h][i] = dout_i w[h]; g_w[h] += sum dout h3; g_b += sum dout
__global__ void k_head_bwd(int n, const float *__restrict__ h3,
                           const float *__restrict__ w,
                           const float *__restrict__ dout,
                           float *__restrict__ dh, float *__restrict__ gw) {
  float acc[H + 1];
#pragma unroll
  for (int h = 0; h <= H; ++h) acc[h] = 0.f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    const float d = dout[i];
#pragma unroll
    for (int h = 0; h < H; ++h) {
      dh[(size_t)h * n + i] = d * w[h];
      acc[h] = fmaf(d, h3[(size_t)h * n + i], acc[h]);
    }
    acc[H] += d;
  }
#pragma unroll
  for (int h = 0; h <= H; ++h) {
    float v = acc[h];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(&gw[h], v);
  }
}

__global__ void k_axpy(int64_t n, const float *__restrict__ x,
                       float *__restrict__ y) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] += x[i];
}

// Adam (Kingma & Ba 2015) on the FP32 master weights
__global__ void k_adam(int n, float *__restrict__ p, const float *__restrict__ g,
                       float *__restrict__ m, float *__restrict__ v, float lr,
                       float b1, float b2, float eps, float c1, float c2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

}  // namespace

struct pg_mpnn {
  Layout lay;
  int64_t n = 0, nnz = 0;
  std::vector<float> host_params;
  pg::DevBuf<float> p, pb, g, m, v;  // master, bf16-rounded, grad, Adam
  pg::DevBuf<int32_t> rp, ci, tr;
  pg::DevBuf<float> feat, r, diag, e, out, dout;
  pg::DevBuf<float> h[L + 1], z[L + 1], q[L], msg[L];
  pg::DevBuf<float> dh, dh2, dz, dq, dmsg;
  pg::DevBuf<double> sums, xg, res, err, st_a, st_b, st_x, st_s;
  pg::DevBuf<double> part;  // per-block partial sums (k_prep, k_loss)
  int step = 0;
  // inference captured as a CUDA graph for one (vals, b, x_prev) address
  // triple; the weights are read from pb at every replay
  cudaGraphExec_t infer = nullptr;
  const double *inf_a = nullptr, *inf_b = nullptr, *inf_x = nullptr;
  int infer_launches = 0;
  ~pg_mpnn() {
    if (infer) cudaGraphExecDestroy(infer);
  }
  void drop_infer() {
    if (infer) cudaGraphExecDestroy(infer);
    infer = nullptr;
  }
};

namespace {

int ensure(pg_mpnn *net, bool training) {
  const int64_t n = net->n, nh = (int64_t)H * n;
  cudaError_t e = cudaSuccess;
  auto rs = [&](auto &buf, size_t cnt) {
    if (e == cudaSuccess) e = buf.reserve(cnt);
  };
  rs(net->feat, (size_t)F * n);
  rs(net->r, n);
  rs(net->diag, n);
  rs(net->e, net->nnz);
  rs(net->out, n);
  rs(net->sums, 16);
  rs(net->part, 4 * (size_t)grid_of(n));
  rs(net->xg, n);
  for (int l = 0; l <= L; ++l) {
    rs(net->h[l], nh);
    rs(net->z[l], nh);
  }
  for (int l = 0; l < L; ++l) {
    rs(net->q[l], nh);
    rs(net->msg[l], nh);
  }
  if (training) {
    rs(net->dout, n);
    rs(net->dh, nh);
    rs(net->dh2, 2 * nh);
    rs(net->dz, nh);
    rs(net->dq, nh);
    rs(net->dmsg, nh);
    rs(net->res, n);
    rs(net->err, n);
  }
  if (e != cudaSuccess) return pg::cuda_fail(e, "mpnn buffers", __FILE__, __LINE__);
  return PG_OK;
}

// forward pass; with `training` it keeps the pre-activations z for the
// backward pass
int forward(pg_mpnn *net, const double *a, const double *b, const double *xp,
            bool training) {
  cudaStream_t st = pg::stream();
  const int n = (int)net->n;
  const int g = grid_of(n);
  const Layout &Y = net->lay;
  const float *W = net->pb.p;
  PG_CUDA(cudaMemsetAsync(net->sums.p, 0, 16 * sizeof(double), st));
  k_prep<<<g, kBlock, 0, st>>>(n, net->rp.p, net->ci.p, a, b, xp, net->r.p,
                               net->diag.p, net->e.p, net->part.p);
  k_finish_sums<<<1, kBlock, 0, st>>>(g, net->part.p, net->sums.p);
  k_features<<<g, kBlock, 0, st>>>(n, b, xp, net->r.p, net->diag.p, net->sums.p,
                                   net->feat.p);
  k_dense_fwd<F, F, H, true, false><<<g, kBlock, 0, st>>>(
      n, net->feat.p, nullptr, W + Y.w0, W + Y.b0, net->h[0].p,
      training ? net->z[0].p : nullptr);
  for (int l = 0; l < L; ++l) {
    k_dense_fwd<H, H, H, false, false><<<g, kBlock, 0, st>>>(
        n, net->h[l].p, nullptr, W + Y.P[l], W + Y.c[l], net->q[l].p, nullptr);
    k_message<<<g, kBlock, 0, st>>>(n, net->rp.p, net->ci.p, net->e.p,
                                    net->q[l].p, net->msg[l].p);
    // h_{l+1} = h_l + relu(U [h_l; m] + d)
    k_dense_fwd<2 * H, H, H, true, true><<<g, kBlock, 0, st>>>(
        n, net->h[l].p, net->msg[l].p, W + Y.U[l], W + Y.d[l],
        net->h[l + 1].p, training ? net->z[l + 1].p : nullptr);
  }
  k_head<<<g, kBlock, 0, st>>>(n, net->h[L].p, W + Y.wo, xp, net->sums.p,
                               net->out.p, net->xg.p);
  pg::count_launches(5 + 3 * L);
  PG_CUDA(cudaGetLastError());
  return PG_OK;
}

// inference forward (fused layers; the guess lands in net->xg): 2 + L + 1
// launches after k_prep / k_finish_sums
int infer_forward(pg_mpnn *net, const double *a, const double *b,
                  const double *xp) {
  cudaStream_t st = pg::stream();
  const int n = (int)net->n;
  const int g = grid_of(n);
  const Layout &Y = net->lay;
  const float *W = net->pb.p;
  PG_CUDA(cudaMemsetAsync(net->sums.p, 0, 16 * sizeof(double), st));
  k_prep<<<g, kBlock, 0, st>>>(n, net->rp.p, net->ci.p, a, b, xp, net->r.p,
                               net->diag.p, net->e.p, net->part.p);
  k_finish_sums<<<1, kBlock, 0, st>>>(g, net->part.p, net->sums.p);
  // h and relu(q) alternate between two buffers each; tiles of kTile cells,
  // a grid of as many CTAs as are resident at once
  static int resident = 0;
  if (!resident) {
    int dev = 0, sms = 0, per_sm = 0;
    PG_CUDA(cudaGetDevice(&dev));
    PG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    PG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
        &per_sm, k_infer_layer<false>, kTileThreads, 0));
    resident = sms * (per_sm > 0 ? per_sm : 1);
  }
  const int tiles = (n + kTile - 1) / kTile;
  const int gt = tiles < resident ? tiles : resident;
  k_infer_in<<<gt, kTileThreads, 0, st>>>(n, b, xp, net->r.p, net->diag.p,
                                   net->sums.p, W + Y.w0, W + Y.b0, W + Y.P[0],
                                   W + Y.c[0], net->h[0].p, net->q[0].p);
  for (int l = 0; l < L; ++l) {
    float *hi = net->h[l & 1].p, *ho = net->h[(l + 1) & 1].p;
    float *qi = net->q[l & 1].p, *qo = net->q[(l + 1) & 1].p;
    if (l + 1 < L)
      k_infer_layer<false><<<gt, kTileThreads, 0, st>>>(
          n, net->rp.p, net->ci.p, net->e.p, qi, hi, W + Y.U[l], W + Y.d[l],
          W + Y.P[l + 1], W + Y.c[l + 1], nullptr, xp, net->sums.p, ho, qo,
          nullptr, nullptr);
    else
      k_infer_layer<true><<<gt, kTileThreads, 0, st>>>(
          n, net->rp.p, net->ci.p, net->e.p, qi, hi, W + Y.U[l], W + Y.d[l],
          nullptr, nullptr, W + Y.wo, xp, net->sums.p, nullptr, nullptr,
          net->out.p, net->xg.p);
  }
  pg::count_launches(3 + L);
  PG_CUDA(cudaGetLastError());
  return PG_OK;
}

int stage_in(const double *src, size_t n, int ptr_kind, pg::DevBuf<double> &buf,
             const double **out) {
  if (ptr_kind == PG_DEVICE) {
    *out = src;
    return PG_OK;
  }
  PG_CUDA(buf.upload(src, n));
  *out = buf.p;
  return PG_OK;
}

}  // namespace

using namespace pg;

extern "C" int pg_mpnn_create(uint64_t seed, pg_mpnn **out) {
  PG_CHECK_ARG(out, "pg_mpnn_create: out is NULL");
  *out = nullptr;
  auto *net = new (std::nothrow) pg_mpnn();
  PG_CHECK_ARG(net, "pg_mpnn_create: out of memory");
  const Layout &Y = net->lay;
  net->host_params.assign(Y.total, 0.f);
  std::mt19937_64 rng(seed);
  auto init = [&](int off, int fan_in, int count) {
    std::normal_distribution<float> d(0.f, std::sqrt(2.f / fan_in));
    for (int i = 0; i < count; ++i) net->host_params[off + i] = d(rng);
  };
  init(Y.w0, F, F * H);
  for (int l = 0; l < L; ++l) {
    init(Y.P[l], H, H * H);
    init(Y.U[l], 2 * H, 2 * H * H);
    // small residual branches at start: the network begins near the
    // previous solution
    for (int i = 0; i < 2 * H * H; ++i) net->host_params[Y.U[l] + i] *= 0.1f;
  }
  // the output head starts at zero: guess = x_prev until trained
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = net->p.upload(net->host_params);
  if (e == cudaSuccess) e = net->pb.reserve(Y.total);
  if (e == cudaSuccess) e = net->g.zero(Y.total);
  if (e == cudaSuccess) e = net->m.zero(Y.total);
  if (e == cudaSuccess) e = net->v.zero(Y.total);
  if (e != cudaSuccess) {
    delete net;
    return cuda_fail(e, "pg_mpnn_create", __FILE__, __LINE__);
  }
  k_round_bf16<<<grid_of(Y.total), kBlock, 0, stream()>>>(Y.total, net->p.p,
                                                         net->pb.p);
  count_launches(1);
  PG_CUDA(cudaStreamSynchronize(stream()));
  *out = net;
  return PG_OK;
}

extern "C" int pg_mpnn_destroy(pg_mpnn *net) {
  if (net) cudaStreamSynchronize(stream());
  delete net;
  return PG_OK;
}

extern "C" int pg_mpnn_num_params(const pg_mpnn *net) {
  return net ? net->lay.total : 0;
}

extern "C" int pg_mpnn_set_graph(pg_mpnn *net, const int32_t *row_ptr,
                                 const int32_t *col_ind, int64_t n) {
  PG_CHECK_ARG(net && row_ptr && col_ind && n > 0, "pg_mpnn_set_graph: bad arg");
  const int64_t nnz = row_ptr[n];
  // transposed entry of every (i, j): the index of (j, i), or -1
  std::vector<int32_t> tr(nnz, -1);
  for (int64_t i = 0; i < n; ++i)
    for (int32_t k = row_ptr[i]; k < row_ptr[i + 1]; ++k) {
      const int32_t j = col_ind[k];
      PG_CHECK_ARG(j >= 0 && j < n, "pg_mpnn_set_graph: column out of range");
      for (int32_t kk = row_ptr[j]; kk < row_ptr[j + 1]; ++kk)
        if (col_ind[kk] == i) {
          tr[k] = kk;
          break;
        }
    }
  net->n = n;
  net->nnz = nnz;
  net->drop_infer();  // buffers may move
  PG_CUDA(net->rp.upload(row_ptr, n + 1));
  PG_CUDA(net->ci.upload(col_ind, nnz));
  PG_CUDA(net->tr.upload(tr));
  int rc = ensure(net, false);
  if (rc) return rc;
  PG_CUDA(cudaStreamSynchronize(stream()));
  return PG_OK;
}

extern "C" int pg_mpnn_predict(pg_mpnn *net, const double *vals,
                               const double *b, const double *x_prev,
                               double *guess, double *rel_residual,
                               int ptr_kind) {
  PG_CHECK_ARG(net && net->n > 0, "pg_mpnn_predict: set the graph first");
  PG_CHECK_ARG(vals && b && x_prev && guess, "pg_mpnn_predict: NULL arg");
  const double *a = nullptr, *bb = nullptr, *xp = nullptr;
  int rc = stage_in(vals, net->nnz, ptr_kind, net->st_a, &a);
  if (!rc) rc = stage_in(b, net->n, ptr_kind, net->st_b, &bb);
  if (!rc) rc = stage_in(x_prev, net->n, ptr_kind, net->st_x, &xp);
  if (!rc) rc = ensure(net, false);
  if (rc) return rc;
  cudaStream_t st = stream();
  const int n = (int)net->n;
  PG_CUDA(net->res.reserve(n));
  // forward + ||b - A g||^2: captured once per input address triple into a
  // CUDA graph and replayed
  auto record = [&]() -> int {
    int r = infer_forward(net, a, bb, xp);
    if (r) return r;
    // ||b - A g||^2 only (no residual vector, no |A x_prev - b|^2)
    k_loss<<<grid_of(n), kBlock, 0, st>>>(n, net->rp.p, net->ci.p, a, bb,
                                         net->xg.p, nullptr, xp, nullptr,
                                         nullptr, net->part.p);
    k_finish_sums<<<1, kBlock, 0, st>>>(grid_of(n), net->part.p, net->sums.p + 4);
    count_launches(2);
    return PG_OK;
  };
  if (!net->infer || net->inf_a != a || net->inf_b != bb || net->inf_x != xp) {
    net->drop_infer();
    cudaGraph_t graph = nullptr;
    const uint64_t before = launch_count();
    PG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
    rc = record();
    cudaError_t ce = cudaStreamEndCapture(st, &graph);
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    PG_CUDA(ce);
    net->infer_launches = (int)(launch_count() - before);
    count_launches(-net->infer_launches);  // counted at each replay
    ce = cudaGraphInstantiate(&net->infer, graph, 0);
    cudaGraphDestroy(graph);
    PG_CUDA(ce);
    net->inf_a = a;
    net->inf_b = bb;
    net->inf_x = xp;
  }
  PG_CUDA(cudaGraphLaunch(net->infer, st));
  count_launches(net->infer_launches);
  if (rel_residual) {  // ||b - A g|| / ||b||
    double s[16];
    PG_CUDA(cudaMemcpyAsync(s, net->sums.p, sizeof(s), cudaMemcpyDeviceToHost, st));
    PG_CUDA(cudaStreamSynchronize(st));
    *rel_residual = s[1] > 0. ? std::sqrt(s[4] / s[1]) : 0.;
  }
  PG_CUDA(copy_out(guess, net->xg.p, net->n * sizeof(double), ptr_kind));
  PG_CUDA(cudaStreamSynchronize(st));
  return PG_OK;
}

// forward + backward: the parameter gradients land in net->g
static int backward_pass(pg_mpnn *net, const double *vals, const double *b,
                         const double *x_prev, const double *x_star,
                         int ptr_kind, double *loss) {
  PG_CHECK_ARG(net && net->n > 0, "pg_mpnn: set the graph first");
  PG_CHECK_ARG(vals && b && x_prev && x_star, "pg_mpnn: NULL arg");
  int rc = ensure(net, true);
  if (rc) return rc;
  const double *a = nullptr, *bb = nullptr, *xp = nullptr, *xs = nullptr;
  rc = stage_in(vals, net->nnz, ptr_kind, net->st_a, &a);
  if (!rc) rc = stage_in(b, net->n, ptr_kind, net->st_b, &bb);
  if (!rc) rc = stage_in(x_prev, net->n, ptr_kind, net->st_x, &xp);
  if (!rc) rc = stage_in(x_star, net->n, ptr_kind, net->st_s, &xs);
  if (!rc) rc = forward(net, a, bb, xp, true);
  if (rc) return rc;
  cudaStream_t st = stream();
  const int n = (int)net->n;
  const int g = grid_of(n);
  const Layout &Y = net->lay;
  const float *W = net->pb.p;
  float *G = net->g.p;
  const size_t nh = (size_t)H * n;
  const int gh = grid_of((int64_t)nh);
  int launches = 0;
  PG_CUDA(cudaMemsetAsync(G, 0, Y.total * sizeof(float), st));
  k_loss<<<g, kBlock, 0, st>>>(n, net->rp.p, net->ci.p, a, bb, net->xg.p, xs,
                               xp, net->res.p, net->err.p, net->part.p);
  k_finish_sums<<<1, kBlock, 0, st>>>(g, net->part.p, net->sums.p + 4);
  ++launches;
  k_dout<<<g, kBlock, 0, st>>>(n, net->rp.p, net->ci.p, net->tr.p, a,
                               net->res.p, net->err.p, net->sums.p,
                               net->dout.p);
  // head: dh = dL/dh_L
  k_head_bwd<<<g, kBlock, 0, st>>>(n, net->h[L].p, W + Y.wo, net->dout.p,
                                   net->dh.p, G + Y.wo);
  launches += 3;
  for (int l = L - 1; l >= 0; --l) {
    // h_{l+1} = h_l + relu(z_{l+1}),  z_{l+1} = U_l [h_l; m_l] + d_l
    k_relu_bwd<<<gh, kBlock, 0, st>>>((int64_t)nh, net->z[l + 1].p, net->dh.p,
                                      net->dz.p);
    k_wgrad<2 * H><<<g, kBlock, 0, st>>>(n, net->h[l].p, H, net->msg[l].p,
                                        net->dz.p, G + Y.U[l], G + Y.d[l]);
    // [dh_l part; dm] = dz U_l^T   (2H outputs)
    k_dense<H, 2 * H, false, false, true><<<g, kBlock, 0, st>>>(
        n, net->dz.p, H, nullptr, W + Y.U[l], nullptr, net->dh2.p, nullptr);
    // m_l = E relu(q_l):  dq = relu'(q_l) (E^T dm)
    k_message_bwd<<<g, kBlock, 0, st>>>(n, net->rp.p, net->ci.p, net->tr.p,
                                        net->e.p, net->q[l].p, net->dh2.p + nh,
                                        net->dq.p);
    k_wgrad<H><<<g, kBlock, 0, st>>>(n, net->h[l].p, H, nullptr, net->dq.p,
                                    G + Y.P[l], G + Y.c[l]);
    // dh_l = dh_{l+1} (residual) + dh2[0:H] + dq P_l^T
    k_axpy<<<gh, kBlock, 0, st>>>((int64_t)nh, net->dh2.p, net->dh.p);
    k_dense<H, H, false, true, true><<<g, kBlock, 0, st>>>(
        n, net->dq.p, H, nullptr, W + Y.P[l], nullptr, net->dh.p, nullptr);
    launches += 7;
  }
  // encoder: h_0 = relu(W0 f + b0)
  k_relu_bwd<<<gh, kBlock, 0, st>>>((int64_t)nh, net->z[0].p, net->dh.p,
                                    net->dz.p);
  k_wgrad<F><<<g, kBlock, 0, st>>>(n, net->feat.p, F, nullptr, net->dz.p,
                                  G + Y.w0, G + Y.b0);
  count_launches(launches + 2);
  PG_CUDA(cudaGetLastError());
  double sm[16];
  PG_CUDA(cudaMemcpyAsync(sm, net->sums.p, sizeof(sm), cudaMemcpyDeviceToHost, st));
  PG_CUDA(cudaStreamSynchronize(st));
  // loss of the forward pass that produced these gradients
  const double lv = (sm[5] > 0. ? sm[4] / sm[5] : 0.) + (sm[7] > 0. ? sm[6] / sm[7] : 0.);
  if (loss) *loss = lv;
  if (!std::isfinite(lv)) {
    set_error("pg_mpnn: non-finite loss");
    return PG_NON_FINITE;
  }
  return PG_OK;
}

extern "C" int pg_mpnn_gradient(pg_mpnn *net, const double *vals,
                                const double *b, const double *x_prev,
                                const double *x_star, int ptr_kind,
                                float *grad, double *loss) {
  int rc = backward_pass(net, vals, b, x_prev, x_star, ptr_kind, loss);
  if (rc) return rc;
  PG_CHECK_ARG(grad, "pg_mpnn_gradient: NULL grad");
  PG_CUDA(cudaMemcpyAsync(grad, net->g.p, net->lay.total * sizeof(float),
                          cudaMemcpyDeviceToHost, stream()));
  PG_CUDA(cudaStreamSynchronize(stream()));
  return PG_OK;
}

extern "C" int pg_mpnn_train_step(pg_mpnn *net, const double *vals,
                                  const double *b, const double *x_prev,
                                  const double *x_star, float lr, int ptr_kind,
                                  double *loss) {
  int rc = backward_pass(net, vals, b, x_prev, x_star, ptr_kind, loss);
  if (rc) return rc;
  cudaStream_t st = stream();
  const Layout &Y = net->lay;
  // Adam on the FP32 master weights, then the BF16-rounded copy
  ++net->step;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, (float)net->step);
  const float c2 = 1.f - std::pow(b2, (float)net->step);
  k_adam<<<grid_of(Y.total), kBlock, 0, st>>>(Y.total, net->p.p, net->g.p, net->m.p,
                                             net->v.p, lr, b1, b2, 1e-8f, c1,
                                             c2);
  k_round_bf16<<<grid_of(Y.total), kBlock, 0, st>>>(Y.total, net->p.p,
                                                   net->pb.p);
  count_launches(2);
  PG_CUDA(cudaGetLastError());
  return PG_OK;
}

extern "C" int pg_mpnn_get_params(const pg_mpnn *net, float *params) {
  PG_CHECK_ARG(net && params, "pg_mpnn_get_params: NULL arg");
  PG_CUDA(cudaMemcpyAsync(params, net->p.p, net->lay.total * sizeof(float),
                          cudaMemcpyDeviceToHost, stream()));
  PG_CUDA(cudaStreamSynchronize(stream()));
  return PG_OK;
}

extern "C" int pg_mpnn_set_params(pg_mpnn *net, const float *params) {
  PG_CHECK_ARG(net && params, "pg_mpnn_set_params: NULL arg");
  const int n = net->lay.total;
  PG_CUDA(net->p.upload(params, n));
  k_round_bf16<<<grid_of(n), kBlock, 0, stream()>>>(n, net->p.p, net->pb.p);
  count_launches(1);
  PG_CUDA(cudaMemsetAsync(net->m.p, 0, n * sizeof(float), stream()));
  PG_CUDA(cudaMemsetAsync(net->v.p, 0, n * sizeof(float), stream()));
  net->step = 0;
  PG_CUDA(cudaStreamSynchronize(stream()));
  return PG_OK;
}

extern "C" int pg_mpnn_save(const pg_mpnn *net, const char *path) {
  PG_CHECK_ARG(net && path, "pg_mpnn_save: NULL arg");
  std::vector<float> p(net->lay.total);
  int rc = pg_mpnn_get_params(net, p.data());
  if (rc) return rc;
  FILE *f = std::fopen(path, "wb");
  PG_CHECK_ARG(f, "pg_mpnn_save: cannot open the file for writing");
  const int32_t n = (int32_t)p.size();
  bool ok = std::fwrite("PGMPNN01", 1, 8, f) == 8 &&
            std::fwrite(&n, sizeof(n), 1, f) == 1 &&
            std::fwrite(p.data(), sizeof(float), p.size(), f) == p.size();
  ok = (std::fclose(f) == 0) && ok;
  PG_CHECK_ARG(ok, "pg_mpnn_save: write failed");
  return PG_OK;
}

extern "C" int pg_mpnn_load(pg_mpnn *net, const char *path) {
  PG_CHECK_ARG(net && path, "pg_mpnn_load: NULL arg");
  FILE *f = std::fopen(path, "rb");
  PG_CHECK_ARG(f, "pg_mpnn_load: cannot open the file");
  char tag[8] = {0};
  int32_t n = 0;
  bool ok = std::fread(tag, 1, 8, f) == 8 && std::memcmp(tag, "PGMPNN01", 8) == 0 &&
            std::fread(&n, sizeof(n), 1, f) == 1 && n == net->lay.total;
  std::vector<float> p(ok ? n : 0);
  if (ok) ok = std::fread(p.data(), sizeof(float), p.size(), f) == p.size();
  std::fclose(f);
  PG_CHECK_ARG(ok, "pg_mpnn_load: not a weights file of this network layout");
  return pg_mpnn_set_params(net, p.data());
}
