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
// as it is applied accurately, which it is (to about 1e-14).  An application is then the K
// subdomain sums of the input (fused into the streamed ILU(0) sweeps), one
// K x K matrix-vector product with a compensated float-float accumulation
// and a constant added to every row of a subdomain.  All reductions run in a fixed order, so
// results are reproducible.
#include <type_traits>

#include "dd.cuh"
#include "kernels.cuh"
#include "lu.h"
#include "../../include/phase_gb300.h"

namespace pg {
namespace {

constexpr int kCoarseBlock = 128;
constexpr int kDefRows = 4;  // rows per thread in flight in k_def_pre
constexpr int kCorrectBlock = 256;
constexpr int kGjB = 32;     // pivots per block of the Gauss-Jordan inversion

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

// the same sums as k_coarse_assemble, kept in FP64 as the values of the
// coarse matrix's CSR (row s: columns cnb[cptr[s] .. cptr[s+1]))
__global__ void __launch_bounds__(kCoarseBlock)
k_coarse_assemble_csr(const int32_t *__restrict__ sub_ptr,
                      const int32_t *__restrict__ prp,
                      const double *__restrict__ val,
                      const int32_t *__restrict__ cptr,
                      const uint8_t *__restrict__ cslot,
                      double *__restrict__ cvals) {
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
    cvals[cptr[s] + j] = sum;
  }
}

// the diagonal before elimination (reference for vanishing pivots)
__global__ void k_gj_diag(int K, const float *__restrict__ ac,
                          float *__restrict__ dg0) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < K) dg0[i] = ac[(size_t)i * K + i];
}

// Blocked Gauss-Jordan inversion in place.  For the pivot block
// k0 .. k0+b-1 with P = A[blk, blk], R = A[blk, :] and C = A[:, blk], b
// single-pivot eliminations amount to
//     A[blk, blk] <- P^-1          A[blk, j] <- (P^-1 R)[:, j]
//     A[i, blk]   <- -(C P^-1)[i]  A[i, j]   <- A[i, j] - C[i, :] (P^-1 R)[:, j]
// (the sweep operator of a block is the product of its pivots' sweeps).

// P^-1 by single-pivot Gauss-Jordan in the registers of one warp: lane q
// holds column q of the pivot block; a pivot below 1e-5 of its original
// diagonal is dropped (its row and column of the inverse are zero).  The
// rows are kept rotated so the pivot row of step k is always c[0] (after
// step k the array shifts by one row), which lets the step loop stay rolled
// (a short loop body instead of 32 unrolled copies) with every register
// index fixed at compile time.  The result goes to pi (shared memory) and,
// to pinv (either may be NULL).
__device__ __forceinline__ void gjb_pivot_block(int K, int k0, int b,
                                                const float *ac,
                                                const float *__restrict__ dg0,
                                                float (*pi)[kGjB + 1],
                                                float *__restrict__ pinv) {
  const int q = threadIdx.x;
  float c[kGjB];
  // read from L2: the block may have been written by this CTA's other
  // warps just before
#pragma unroll
  for (int p = 0; p < kGjB; ++p)
    c[p] = p < b && q < b ? __ldcg(ac + (size_t)(k0 + p) * K + k0 + q) : 0.f;
  // the original diagonal of the block: lane q holds pivot q's, read once
  const float d0 = q < b ? fabsf(dg0[k0 + q]) : 0.f;
#pragma unroll 1
  for (int k = 0; k < b; ++k) {
    // c[p] holds row (k + p) mod 32
    const float piv = __shfl_sync(0xffffffffu, c[0], k);
    const float dk = __shfl_sync(0xffffffffu, d0, k);
    const float ip = fabsf(piv) > 1e-5f * dk ? 1.f / piv : 0.f;
    const float rk = c[0];  // P[k][q]
    c[0] = q == k ? ip : rk * ip;
#pragma unroll
    for (int p = 1; p < kGjB; ++p) {
      const float cpk = __shfl_sync(0xffffffffu, c[p], k);  // P[k+p][k]
      c[p] = q == k ? -cpk * ip : c[p] - cpk * (rk * ip);
    }
    const float t0 = c[0];
#pragma unroll
    for (int p = 0; p + 1 < kGjB; ++p) c[p] = c[p + 1];
    c[kGjB - 1] = t0;
  }
  // after b steps c[p] holds row (b + p) mod 32
#pragma unroll
  for (int p = 0; p < kGjB; ++p) {
    const int row = (b + p) & (kGjB - 1);
    if (pi) pi[row][q] = c[p];
    if (pinv) pinv[row * kGjB + q] = c[p];
  }
}

// W = P^-1 R (b x K) and V = C P^-1 (K x b); C is kept (K x b) for the
// update, which overwrites the block columns.  Blocks [0, nw): 32 columns
// of W each (thread (x, y): column x, rows y, y+8, ...); blocks after:
// rows of V and C (four threads per row, eight columns each).
__global__ void __launch_bounds__(256)
k_gjb_panel(int K, int k0, int b, int nw, const float *__restrict__ ac,
            const float *__restrict__ dg0, float *__restrict__ pinv,
            int invert, float *__restrict__ W, float *__restrict__ V,
            float *__restrict__ C) {
  pdl_wait();
  // the pivot block's inverse: the previous step's update computed it
  // (pinv), except on the first step, where every CTA inverts the block
  // itself (one warp) and the first one stores it; the CTA's own operands
  // are read first, in flight meanwhile
  __shared__ float pi[kGjB][kGjB + 1];
  const bool wpart = (int)blockIdx.x < nw;
  const int t = wpart ? 0 : ((int)blockIdx.x - nw) * 256 + (int)threadIdx.x;
  const int j = wpart ? (int)blockIdx.x * 32 + (int)(threadIdx.x & 31) : 0;
  const int i = t >> 2, p0 = (t & 3) * 8;
  const bool live = wpart ? j < K : i < K;
  float r[kGjB];  // W part: column j of R; V part: row i of C
#pragma unroll
  for (int q = 0; q < kGjB; ++q)
    r[q] = live && q < b ? (wpart ? ac[(size_t)(k0 + q) * K + j]
                                  : ac[(size_t)i * K + k0 + q])
                         : 0.f;
  if (invert) {
    if (threadIdx.x < 32)
      gjb_pivot_block(K, k0, b, ac, dg0, pi, blockIdx.x == 0 ? pinv : nullptr);
  } else {
    for (int e = threadIdx.x; e < kGjB * kGjB; e += 256)
      pi[e / kGjB][e % kGjB] = pinv[e];
  }
  __syncthreads();
  if (!live) return;
  if (wpart) {
    for (int p = threadIdx.x >> 5; p < b; p += 8) {
      float acc = 0.f;
#pragma unroll
      for (int q = 0; q < kGjB; ++q) acc += pi[p][q] * r[q];
      W[(size_t)p * K + j] = acc;
    }
  } else {
#pragma unroll
    for (int pp = 0; pp < 8; ++pp) {
      const int p = p0 + pp;
      float acc = 0.f;
#pragma unroll
      for (int q = 0; q < kGjB; ++q) acc += r[q] * pi[q][p];
      V[(size_t)i * kGjB + p] = acc;
      C[(size_t)i * kGjB + p] = p < b ? ac[(size_t)i * K + k0 + p] : 0.f;
    }
  }
}

// The update of every entry, register-tiled: a CTA owns a kUpdRows x
// kUpdCols tile; the pivot block's rows of C (transposed, 32 x kUpdRows) and
// columns of W (32 x kUpdCols) are staged in shared memory, and each thread
// keeps 4 rows x 4 consecutive columns of sums in registers, reading its 4
// W values and its 4 C values with one 16-byte load each per pivot (a warp
// shares its rows, so its C loads are broadcasts).  The tile's entries of A
// are read at the start, all in flight together (16-byte accesses when
// every row of A is 16-byte aligned, VEC), and each sum runs over the 32
// pivots in order, as C[i, :] . W[:, j] with zeros past b.
constexpr int kUpdRows = 32, kUpdCols = 128;
template <bool VEC>
__global__ void __launch_bounds__(256, 4)
k_gjb_update(int K, int k0, int b, float *ac, const float *__restrict__ pinv,
             const float *__restrict__ dg0, float *__restrict__ pinv_next,
             const float *__restrict__ W, const float *__restrict__ V,
             const float *__restrict__ C) {
  pdl_wait();
  __shared__ __align__(16) float ws[kGjB][kUpdCols];
  __shared__ __align__(16) float ct[kGjB][kUpdRows];
  // The tile holding the next pivot block (rows and columns k0+32 ..
  // k0+63) is given to the first CTA, which afterwards inverts that block
  // for the next step's panel while the other tiles are being updated.
  const int k1 = k0 + kGjB;
  const int tiles_x = gridDim.x, n_tiles = gridDim.x * gridDim.y;
  const int own = k1 < K ? (k1 / kUpdRows) * tiles_x + k1 / kUpdCols : 0;
  const int tile = ((int)(blockIdx.y * gridDim.x + blockIdx.x) + own) % n_tiles;
  const int j0 = (tile % tiles_x) * kUpdCols, i0 = (tile / tiles_x) * kUpdRows;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  const int jt = j0 + 4 * tx;  // this thread's first column
  float a_old[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int i = i0 + ty * 4 + r;
    if (VEC && i < K && jt + 3 < K) {
      const float4 x = *reinterpret_cast<const float4 *>(ac + (size_t)i * K + jt);
      a_old[r][0] = x.x, a_old[r][1] = x.y, a_old[r][2] = x.z, a_old[r][3] = x.w;
    } else {
#pragma unroll
      for (int c = 0; c < 4; ++c)
        a_old[r][c] = i < K && jt + c < K ? ac[(size_t)i * K + jt + c] : 0.f;
    }
  }
  // W and C tiles: every load is issued before the first store to shared
  // memory, so the tile arrives in one round trip
  {
    constexpr int NW = kGjB * kUpdCols / 4 / 256;  // 16-byte pieces per thread
    float4 wl[NW];
#pragma unroll
    for (int u = 0; u < NW; ++u) {
      const int e = threadIdx.x + 256 * u;
      const int q = e / (kUpdCols / 4), jj = j0 + 4 * (e % (kUpdCols / 4));
      const float *src = W + (size_t)q * K + jj;
      if (VEC && q < b && jj + 3 < K) {
        wl[u] = *reinterpret_cast<const float4 *>(src);
      } else {
        wl[u].x = q < b && jj < K ? src[0] : 0.f;
        wl[u].y = q < b && jj + 1 < K ? src[1] : 0.f;
        wl[u].z = q < b && jj + 2 < K ? src[2] : 0.f;
        wl[u].w = q < b && jj + 3 < K ? src[3] : 0.f;
      }
    }
    // C rows are 32 contiguous floats (16-byte aligned): thread e takes row
    // e / 8, pivots 4 (e % 8) .. +3
    const int ii = i0 + threadIdx.x / 8, q4 = 4 * (threadIdx.x % 8);
    float4 cl = make_float4(0.f, 0.f, 0.f, 0.f);
    if (ii < K) cl = *reinterpret_cast<const float4 *>(C + (size_t)ii * kGjB + q4);
#pragma unroll
    for (int u = 0; u < NW; ++u) {
      const int e = threadIdx.x + 256 * u;
      *reinterpret_cast<float4 *>(&ws[e / (kUpdCols / 4)][4 * (e % (kUpdCols / 4))]) = wl[u];
    }
    ct[q4][threadIdx.x / 8] = cl.x;
    ct[q4 + 1][threadIdx.x / 8] = cl.y;
    ct[q4 + 2][threadIdx.x / 8] = cl.z;
    ct[q4 + 3][threadIdx.x / 8] = cl.w;
  }
  __syncthreads();
  float acc[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[r][c] = 0.f;
#pragma unroll 8
  for (int q = 0; q < kGjB; ++q) {
    const float4 w = *reinterpret_cast<const float4 *>(&ws[q][4 * tx]);
    const float4 cv = *reinterpret_cast<const float4 *>(&ct[q][4 * ty]);
    const float wv[4] = {w.x, w.y, w.z, w.w}, cr[4] = {cv.x, cv.y, cv.z, cv.w};
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int c = 0; c < 4; ++c) acc[r][c] += cr[r] * wv[c];
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int i = i0 + ty * 4 + r;
    if (i >= K) break;
    const bool iin = i >= k0 && i < k0 + b;
    float v[4];
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int j = jt + c;
      const bool jin = j >= k0 && j < k0 + b;
      if (iin && jin)
        v[c] = pinv[(i - k0) * kGjB + (j - k0)];
      else if (iin)
        v[c] = ws[i - k0][4 * tx + c];
      else if (jin)
        v[c] = -V[(size_t)i * kGjB + (j - k0)];
      else
        v[c] = a_old[r][c] - acc[r][c];
    }
    if (VEC && jt + 3 < K) {
      *reinterpret_cast<float4 *>(ac + (size_t)i * K + jt) =
          make_float4(v[0], v[1], v[2], v[3]);
    } else {
#pragma unroll
      for (int c = 0; c < 4; ++c)
        if (jt + c < K) ac[(size_t)i * K + jt + c] = v[c];
    }
  }
  if (k1 < K && blockIdx.x == 0 && blockIdx.y == 0) {
    __threadfence();  // this CTA's entries of A are in L2 ...
    __syncthreads();  // ... for every warp
    if (threadIdx.x < 32)
      gjb_pivot_block(K, k1, K - k1 < kGjB ? K - k1 : kGjB, ac, dg0, nullptr,
                      pinv_next);
  }
}

// Z^T in: one sum per subdomain, stored as a float pair (hi + lo)
__global__ void __launch_bounds__(kCoarseBlock)
k_coarse_sum(const int32_t *__restrict__ sub_ptr, const double *__restrict__ in,
             float2 *__restrict__ csum, const KScalars *__restrict__ sc) {
  if (sc && sc->done) return;
  __shared__ double red[kCoarseBlock];
  const int s = blockIdx.x;
  double acc = 0.;
  for (int32_t i = sub_ptr[s] + threadIdx.x; i < sub_ptr[s + 1]; i += kCoarseBlock)
    acc += in[i];
  const double t = block_sum(acc, red);
  if (threadIdx.x == 0) csum[s] = dd_from(t);
}

__global__ void __launch_bounds__(kCoarseBlock)
k_coarse_sum_dd(const int32_t *__restrict__ sub_ptr,
                const float2 *__restrict__ in, float2 *__restrict__ csum,
                const KScalars *__restrict__ sc) {
  if (sc && sc->done) return;
  __shared__ double red[kCoarseBlock];
  const int s = blockIdx.x;
  DdAcc acc = dd_acc(make_float2(0.f, 0.f));
  for (int32_t i = sub_ptr[s] + threadIdx.x; i < sub_ptr[s + 1]; i += kCoarseBlock)
    dd_acc_add(acc, in[i]);
  const double t = block_sum(dd_acc_to_double(acc), red);
  if (threadIdx.x == 0) csum[s] = dd_from(t);
}

// y_s = (A_c^-1)_s . csum with a compensated float-float accumulation on
// the FP32 pipes (the FP32 inverse entries times the float-pair sums:
// TwoProduct of the high parts plus the low-part product; about 1e-14
// relative, so the correction stays a linear operator to that level), then
// z += y_s on the rows of subdomain s (one CTA per subdomain)
template <class VT>
__global__ void __launch_bounds__(kCorrectBlock)
k_coarse_correct(int K, const int32_t *__restrict__ sub_ptr,
                 const float *__restrict__ ainv,
                 const float2 *__restrict__ csum, VT *__restrict__ z,
                 const KScalars *__restrict__ sc) {
  if (sc && sc->done) return;
  __shared__ float red_s[kCorrectBlock / 32], red_c[kCorrectBlock / 32];
  __shared__ double y_sh;
  const int s = blockIdx.x;
  const float *row = ainv + (size_t)s * K;
  DdAcc acc = dd_acc(make_float2(0.f, 0.f));
  for (int j = threadIdx.x; j < K; j += kCorrectBlock)
    dd_acc_fma(acc, make_float2(row[j], 0.f), csum[j]);
  // fixed-order reduction: butterfly within the warp, then warp order
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    DdAcc b;
    b.s = __shfl_xor_sync(0xffffffffu, acc.s, o);
    b.c = __shfl_xor_sync(0xffffffffu, acc.c, o);
    dd_acc_merge(acc, b);
  }
  const int wid = threadIdx.x / 32;
  if ((threadIdx.x & 31) == 0) {
    red_s[wid] = acc.s;
    red_c[wid] = acc.c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    DdAcc t = dd_acc(make_float2(red_s[0], red_c[0]));
    for (int w = 1; w < kCorrectBlock / 32; ++w) {
      DdAcc b;
      b.s = red_s[w];
      b.c = red_c[w];
      dd_acc_merge(t, b);
    }
    y_sh = dd_acc_to_double(t);
  }
  __syncthreads();
  const double y = y_sh;
  if constexpr (std::is_same<VT, double>::value) {
    for (int32_t i = sub_ptr[s] + threadIdx.x; i < sub_ptr[s + 1]; i += kCorrectBlock)
      z[i] += y;
  } else {
    const float2 yd = dd_from(y);
    for (int32_t i = sub_ptr[s] + threadIdx.x; i < sub_ptr[s + 1]; i += kCorrectBlock)
      z[i] = dd_add(z[i], yd);
  }
}

// ------------------------------------------------ deflated application
// A-DEF1 (Tang, Nabben, Vuik & Erlangga, J. Sci. Comput. 39, 2009):
//     M^-1 r = B (r - A Z y) + Z y,   y = A_c^-1 Z^T r,
// B the Schwarz ILU(0) sweeps.  A Z is kept per row as the sums of the
// row's entries over each subdomain its columns fall in.  One application:
// k_def_pre (the Krylov update of the input and its subdomain sums),
// k_coarse_y (y), k_def_in (r - A Z y), then the sweep; the streamed sweep
// adds Z y as it writes z (its mode 3), k_coarse_add does it after the
// other sweep forms.

// (A Z) values from the permuted matrix, row by row in entry order
__global__ void k_az_values(int n, const int32_t *__restrict__ prp,
                            const int32_t *__restrict__ azp,
                            const uint8_t *__restrict__ azslot,
                            const double *__restrict__ val,
                            double *__restrict__ azv) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    for (int32_t q = azp[i]; q < azp[i + 1]; ++q) azv[q] = 0.;
    for (int32_t k = prp[i]; k < prp[i + 1]; ++k) azv[azp[i] + azslot[k]] += val[k];
  }
}

// the preconditioner's input with the fused BiCGStab update (written back
// to pv) and its subdomain sums (one CTA per subdomain)
__global__ void __launch_bounds__(kCoarseBlock)
k_def_pre(int mode, const int32_t *__restrict__ sub_ptr,
          const double *__restrict__ r, double *__restrict__ pv,
          const double *__restrict__ v, const KScalars *__restrict__ sc,
          float2 *__restrict__ csum) {
  pdl_wait();
  if (sc && sc->done) return;
  __shared__ double red[kCoarseBlock];
  const int s = blockIdx.x;
  double acc = 0.;
  const int32_t e = sub_ptr[s + 1];
  for (int32_t i0 = sub_ptr[s] + threadIdx.x; i0 < e; i0 += kDefRows * kCoarseBlock) {
    // the group's loads first, then the rows in order
    double ri[kDefRows], pi[kDefRows], vi[kDefRows];
#pragma unroll
    for (int u = 0; u < kDefRows; ++u) {
      const int32_t i = i0 + u * kCoarseBlock;
      const bool in = i < e;
      ri[u] = in && mode ? r[i] : 0.;
      pi[u] = in && mode != 2 ? pv[i] : 0.;
      vi[u] = in && mode ? v[i] : 0.;
    }
#pragma unroll
    for (int u = 0; u < kDefRows; ++u) {
      const int32_t i = i0 + u * kCoarseBlock;
      if (i < e) {
        const double val = pre_combine<double>(mode, ri[u], pi[u], vi[u], sc);
        if (mode) pv[i] = val;
        acc += val;
      }
    }
  }
  const double t = block_sum(acc, red);
  if (threadIdx.x == 0) csum[s] = dd_from(t);
}

// y_s = (A_c^-1)_s . csum (compensated float-float dot, as k_coarse_correct);
// y_dd (optional) receives y as float pairs for the float-float solver
__global__ void __launch_bounds__(kCorrectBlock)
k_coarse_y(int K, const float *__restrict__ ainv,
           const float2 *__restrict__ csum, double *__restrict__ y,
           float2 *__restrict__ y_dd, const KScalars *__restrict__ sc) {
  pdl_wait();
  if (sc && sc->done) return;
  __shared__ float red_s[kCorrectBlock / 32], red_c[kCorrectBlock / 32];
  const int s = blockIdx.x;
  const float *row = ainv + (size_t)s * K;
  DdAcc acc = dd_acc(make_float2(0.f, 0.f));
  for (int j = threadIdx.x; j < K; j += kCorrectBlock)
    dd_acc_fma(acc, make_float2(row[j], 0.f), csum[j]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    DdAcc b;
    b.s = __shfl_xor_sync(0xffffffffu, acc.s, o);
    b.c = __shfl_xor_sync(0xffffffffu, acc.c, o);
    dd_acc_merge(acc, b);
  }
  const int wid = threadIdx.x / 32;
  if ((threadIdx.x & 31) == 0) {
    red_s[wid] = acc.s;
    red_c[wid] = acc.c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    DdAcc u = dd_acc(make_float2(red_s[0], red_c[0]));
    for (int w = 1; w < kCorrectBlock / 32; ++w) {
      DdAcc b;
      b.s = red_s[w];
      b.c = red_c[w];
      dd_acc_merge(u, b);
    }
    const double v = dd_acc_to_double(u);
    y[s] = v;
    if (y_dd) y_dd[s] = dd_from(v);
  }
}

// t = pv - (A Z) y
__global__ void k_def_in(int n, const int32_t *__restrict__ azp,
                         const int32_t *__restrict__ azj,
                         const double *__restrict__ azv,
                         const double *__restrict__ y,
                         const double *__restrict__ pv, double *__restrict__ t,
                         const KScalars *__restrict__ sc) {
  pdl_wait();
  if (sc && sc->done) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    double acc = pv[i];
    for (int32_t q = azp[i]; q < azp[i + 1]; ++q) acc -= azv[q] * y[azj[q]];
    t[i] = acc;
  }
}

// z += y_s on the rows of subdomain s
__global__ void __launch_bounds__(kCorrectBlock)
k_coarse_add(const int32_t *__restrict__ sub_ptr, const double *__restrict__ y,
             double *__restrict__ z, const KScalars *__restrict__ sc) {
  if (sc && sc->done) return;
  const int s = blockIdx.x;
  const double ys = y[s];
  for (int32_t i = sub_ptr[s] + threadIdx.x; i < sub_ptr[s + 1]; i += kCorrectBlock)
    z[i] += ys;
}

// float-float forms of the deflated application (the mixed solver)
__global__ void __launch_bounds__(kCoarseBlock)
k_def_pre_dd(int mode, const int32_t *__restrict__ sub_ptr,
             const float2 *__restrict__ r, float2 *__restrict__ pv,
             const float2 *__restrict__ v, const KScalars *__restrict__ sc,
             float2 *__restrict__ csum) {
  pdl_wait();
  if (sc && sc->done) return;
  __shared__ double red[kCoarseBlock];
  const int s = blockIdx.x;
  const float2 zero = make_float2(0.f, 0.f);
  DdAcc acc = dd_acc(zero);
  const int32_t e = sub_ptr[s + 1];
  for (int32_t i0 = sub_ptr[s] + threadIdx.x; i0 < e; i0 += kDefRows * kCoarseBlock) {
    // the group's loads first, then the rows in order
    float2 ri[kDefRows], pi[kDefRows], vi[kDefRows];
#pragma unroll
    for (int u = 0; u < kDefRows; ++u) {
      const int32_t i = i0 + u * kCoarseBlock;
      const bool in = i < e;
      ri[u] = in && mode ? r[i] : zero;
      pi[u] = in && mode != 2 ? pv[i] : zero;
      vi[u] = in && mode ? v[i] : zero;
    }
#pragma unroll
    for (int u = 0; u < kDefRows; ++u) {
      const int32_t i = i0 + u * kCoarseBlock;
      if (i < e) {
        const float2 val = dd_pre_combine(mode, ri[u], pi[u], vi[u], sc);
        if (mode) pv[i] = val;
        dd_acc_add(acc, val);
      }
    }
  }
  const double t = block_sum(dd_acc_to_double(acc), red);
  if (threadIdx.x == 0) csum[s] = dd_from(t);
}

// t = pv - (A Z) y in float-float
__global__ void k_def_in_dd(int n, const int32_t *__restrict__ azp,
                            const int32_t *__restrict__ azj,
                            const float2 *__restrict__ azv,
                            const float2 *__restrict__ y,
                            const float2 *__restrict__ pv,
                            float2 *__restrict__ t,
                            const KScalars *__restrict__ sc) {
  pdl_wait();
  if (sc && sc->done) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += gridDim.x * blockDim.x) {
    DdAcc acc = dd_acc(pv[i]);
    for (int32_t q = azp[i]; q < azp[i + 1]; ++q)
      dd_acc_fma(acc, dd_neg(azv[q]), y[azj[q]]);
    t[i] = dd_value(acc);
  }
}

__global__ void __launch_bounds__(kCorrectBlock)
k_coarse_add_dd(const int32_t *__restrict__ sub_ptr,
                const float2 *__restrict__ y, float2 *__restrict__ z,
                const KScalars *__restrict__ sc) {
  if (sc && sc->done) return;
  const int s = blockIdx.x;
  const float2 ys = y[s];
  for (int32_t i = sub_ptr[s] + threadIdx.x; i < sub_ptr[s + 1]; i += kCorrectBlock)
    z[i] = dd_add(z[i], ys);
}

// ------------------------------------------------------ batched systems
// Block-diagonal coarse space of stacked independent systems: system t owns
// subdomains [k0[t], k0[t+1]) and a dense K_t x K_t block of A_c at float
// offset off[t]; nothing couples systems.

__global__ void __launch_bounds__(kCoarseBlock)
k_coarse_assemble_b(CoarseBatchDev c, const int32_t *__restrict__ prp,
                    const double *__restrict__ val) {
  extern __shared__ double part[];  // [kCoarseBlock][S]
  const int s = blockIdx.x;
  const int t = c.sub_sys[s];
  const int k0 = c.k0[t], Kt = c.k0[t + 1] - k0;
  const int S = c.cptr[s + 1] - c.cptr[s];
  for (int j = 0; j < S; ++j) part[threadIdx.x * S + j] = 0.;
  const int32_t e0 = prp[c.sub_ptr[s]], e1 = prp[c.sub_ptr[s + 1]];
  for (int32_t k = e0 + threadIdx.x; k < e1; k += kCoarseBlock)
    part[threadIdx.x * S + c.cslot[k]] += val[k];
  __syncthreads();
  float *blk = c.ac + c.off[t] + (size_t)(s - k0) * Kt;
  for (int j = threadIdx.x; j < S; j += kCoarseBlock) {
    double sum = 0.;
    for (int q = 0; q < kCoarseBlock; ++q) sum += part[q * S + j];
    blk[c.cnb[c.cptr[s] + j] - k0] = (float)sum;
  }
}

// Gauss-Jordan inversion of one system's block in place by one CTA of
// 32 x 32 threads (single pivots, the same arithmetic as the blocked form;
// a pivot below 1e-5 of its original diagonal is dropped)
__global__ void __launch_bounds__(1024)
k_gj_block(CoarseBatchDev c) {
  extern __shared__ float sm[];  // dg0 | rowk | colk, max_k each
  const int t = blockIdx.x;
  const int Kt = c.k0[t + 1] - c.k0[t];
  float *a = c.ac + c.off[t];
  float *dg0 = sm, *rowk = sm + c.max_k, *colk = sm + 2 * c.max_k;
  const int tid = threadIdx.x, tx = tid & 31, ty = tid >> 5;
  for (int i = tid; i < Kt; i += 1024) dg0[i] = a[(size_t)i * Kt + i];
  for (int k = 0; k < Kt; ++k) {
    __syncthreads();  // the previous step's writes are done
    for (int j = tid; j < Kt; j += 1024) {
      rowk[j] = a[(size_t)k * Kt + j];
      colk[j] = a[(size_t)j * Kt + k];
    }
    __syncthreads();
    const float piv = rowk[k];
    const float ip = fabsf(piv) > 1e-5f * fabsf(dg0[k]) ? 1.f / piv : 0.f;
    for (int i = ty; i < Kt; i += 32) {
      const float a_ik = colk[i];
      for (int j = tx; j < Kt; j += 32) {
        const size_t idx = (size_t)i * Kt + j;
        const float a_kj = rowk[j];
        float v;
        if (i == k && j == k)
          v = ip;
        else if (i == k)
          v = a_kj * ip;
        else if (j == k)
          v = -a_ik * ip;
        else
          v = a[idx] - a_ik * (a_kj * ip);
        a[idx] = v;
      }
    }
  }
}

// per-subdomain input sums of the systems still running
__global__ void __launch_bounds__(kCoarseBlock)
k_coarse_sum_b(CoarseBatchDev c, const double *__restrict__ in,
               const KScalars *__restrict__ sc) {
  const int s = blockIdx.x;
  if (sc[c.sub_sys[s]].done) return;
  __shared__ double red[kCoarseBlock];
  double acc = 0.;
  for (int32_t i = c.sub_ptr[s] + threadIdx.x; i < c.sub_ptr[s + 1]; i += kCoarseBlock)
    acc += in[i];
  const double t = block_sum(acc, red);
  if (threadIdx.x == 0) c.csum[s] = dd_from(t);
}

// y_s = (A_t^-1)_s . csum over the system's subdomains, z += y_s
__global__ void __launch_bounds__(kCorrectBlock)
k_coarse_correct_b(CoarseBatchDev c, double *__restrict__ z,
                   const KScalars *__restrict__ sc) {
  const int s = blockIdx.x;
  const int t = c.sub_sys[s];
  if (sc[t].done) return;
  __shared__ float red_s[kCorrectBlock / 32], red_c[kCorrectBlock / 32];
  __shared__ double y_sh;
  const int k0 = c.k0[t], Kt = c.k0[t + 1] - k0;
  const float *row = c.ac + c.off[t] + (size_t)(s - k0) * Kt;
  DdAcc acc = dd_acc(make_float2(0.f, 0.f));
  for (int j = threadIdx.x; j < Kt; j += kCorrectBlock)
    dd_acc_fma(acc, make_float2(row[j], 0.f), c.csum[k0 + j]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    DdAcc b;
    b.s = __shfl_xor_sync(0xffffffffu, acc.s, o);
    b.c = __shfl_xor_sync(0xffffffffu, acc.c, o);
    dd_acc_merge(acc, b);
  }
  const int wid = threadIdx.x / 32;
  if ((threadIdx.x & 31) == 0) {
    red_s[wid] = acc.s;
    red_c[wid] = acc.c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    DdAcc u = dd_acc(make_float2(red_s[0], red_c[0]));
    for (int w = 1; w < kCorrectBlock / 32; ++w) {
      DdAcc b;
      b.s = red_s[w];
      b.c = red_c[w];
      dd_acc_merge(u, b);
    }
    y_sh = dd_acc_to_double(u);
  }
  __syncthreads();
  const double y = y_sh;
  for (int32_t i = c.sub_ptr[s] + threadIdx.x; i < c.sub_ptr[s + 1]; i += kCorrectBlock)
    z[i] += y;
}

// deflated application for batches: one CTA per subdomain, the scalars of
// its system (done systems skip)
__global__ void __launch_bounds__(kCoarseBlock)
k_def_pre_b(int mode, CoarseBatchDev c, const double *__restrict__ r,
            double *__restrict__ pv, const double *__restrict__ v,
            const KScalars *__restrict__ sc_base) {
  const int s = blockIdx.x;
  const KScalars *sc = sc_base + c.sub_sys[s];
  if (sc->done) return;
  __shared__ double red[kCoarseBlock];
  double acc = 0.;
  for (int32_t i = c.sub_ptr[s] + threadIdx.x; i < c.sub_ptr[s + 1]; i += kCoarseBlock) {
    const double val = pre_combine<double>(mode, mode ? r[i] : 0.,
                                           mode != 2 ? pv[i] : 0.,
                                           mode ? v[i] : 0., sc);
    if (mode) pv[i] = val;
    acc += val;
  }
  const double t = block_sum(acc, red);
  if (threadIdx.x == 0) c.csum[s] = dd_from(t);
}

__global__ void __launch_bounds__(kCorrectBlock)
k_coarse_y_b(CoarseBatchDev c, const KScalars *__restrict__ sc) {
  const int s = blockIdx.x;
  const int t = c.sub_sys[s];
  if (sc[t].done) return;
  __shared__ float red_s[kCorrectBlock / 32], red_c[kCorrectBlock / 32];
  const int k0 = c.k0[t], Kt = c.k0[t + 1] - k0;
  const float *row = c.ac + c.off[t] + (size_t)(s - k0) * Kt;
  DdAcc acc = dd_acc(make_float2(0.f, 0.f));
  for (int j = threadIdx.x; j < Kt; j += kCorrectBlock)
    dd_acc_fma(acc, make_float2(row[j], 0.f), c.csum[k0 + j]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    DdAcc b;
    b.s = __shfl_xor_sync(0xffffffffu, acc.s, o);
    b.c = __shfl_xor_sync(0xffffffffu, acc.c, o);
    dd_acc_merge(acc, b);
  }
  const int wid = threadIdx.x / 32;
  if ((threadIdx.x & 31) == 0) {
    red_s[wid] = acc.s;
    red_c[wid] = acc.c;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    DdAcc u = dd_acc(make_float2(red_s[0], red_c[0]));
    for (int w = 1; w < kCorrectBlock / 32; ++w) {
      DdAcc b;
      b.s = red_s[w];
      b.c = red_c[w];
      dd_acc_merge(u, b);
    }
    c.y[s] = dd_acc_to_double(u);
  }
}

__global__ void __launch_bounds__(kCorrectBlock)
k_def_in_b(CoarseBatchDev c, const double *__restrict__ pv,
           double *__restrict__ tmp, const KScalars *__restrict__ sc) {
  const int s = blockIdx.x;
  if (sc[c.sub_sys[s]].done) return;
  for (int32_t i = c.sub_ptr[s] + threadIdx.x; i < c.sub_ptr[s + 1]; i += kCorrectBlock) {
    double acc = pv[i];
    for (int32_t q = c.azp[i]; q < c.azp[i + 1]; ++q) acc -= c.azv[q] * c.y[c.azj[q]];
    tmp[i] = acc;
  }
}

__global__ void __launch_bounds__(kCorrectBlock)
k_coarse_add_b(CoarseBatchDev c, double *__restrict__ z,
               const KScalars *__restrict__ sc) {
  const int s = blockIdx.x;
  if (sc[c.sub_sys[s]].done) return;
  const double ys = c.y[s];
  for (int32_t i = c.sub_ptr[s] + threadIdx.x; i < c.sub_ptr[s + 1]; i += kCorrectBlock)
    z[i] += ys;
}

}  // namespace

void launch_def_pre_b(const CoarseBatchDev &c, int K, int mode, const double *r,
                      double *pv, const double *v, double *tmp,
                      const KScalars *sc, cudaStream_t st) {
  k_def_pre_b<<<K, kCoarseBlock, 0, st>>>(mode, c, r, pv, v, sc);
  k_coarse_y_b<<<K, kCorrectBlock, 0, st>>>(c, sc);
  k_def_in_b<<<K, kCorrectBlock, 0, st>>>(c, pv, tmp, sc);
  count_launches(3);
}

void launch_coarse_add_b(const CoarseBatchDev &c, int K, double *z,
                         const KScalars *sc, cudaStream_t st) {
  k_coarse_add_b<<<K, kCorrectBlock, 0, st>>>(c, z, sc);
  count_launches(1);
}

void launch_az_values(const CoarseDev &c, int n, const int32_t *prp,
                      const double *pvals, cudaStream_t st) {
  const int g = (n + 255) / 256 < 2432 ? (n + 255) / 256 : 2432;
  k_az_values<<<g, 256, 0, st>>>(n, prp, c.azp, c.azslot, pvals, c.azv);
  count_launches(1);
}

void launch_def_pre(const CoarseDev &c, int mode, const double *r, double *pv,
                    const double *v, const KScalars *sc, cudaStream_t st) {
  launch_pdl(k_def_pre, c.K, kCoarseBlock, 0, st, mode, c.sub_ptr, r, pv, v, sc, c.csum);
  launch_pdl(k_coarse_y, c.K, kCorrectBlock, 0, st, c.K, (const float *)c.ac, (const float2 *)c.csum, c.y, (float2 *)nullptr, sc);
  count_launches(2);
}

void launch_def_in(const CoarseDev &c, int n, const double *pv, double *t,
                   const KScalars *sc, cudaStream_t st) {
  const int g = (n + 255) / 256 < 2432 ? (n + 255) / 256 : 2432;
  launch_pdl(k_def_in, g, 256, 0, st, n, c.azp, c.azj, c.azv, c.y, pv, t, sc);
  count_launches(1);
}

void launch_coarse_add(const CoarseDev &c, double *z, const KScalars *sc,
                       cudaStream_t st) {
  k_coarse_add<<<c.K, kCorrectBlock, 0, st>>>(c.sub_ptr, c.y, z, sc);
  count_launches(1);
}

void launch_def_pre_dd(const CoarseDev &c, int mode, const float2 *r,
                       float2 *pv, const float2 *v, const KScalars *sc,
                       cudaStream_t st) {
  launch_pdl(k_def_pre_dd, c.K, kCoarseBlock, 0, st, mode, c.sub_ptr, r, pv, v, sc, c.csum);
  launch_pdl(k_coarse_y, c.K, kCorrectBlock, 0, st, c.K, (const float *)c.ac, (const float2 *)c.csum, c.y, c.y_dd, sc);
  count_launches(2);
}

void launch_def_in_dd(const CoarseDev &c, int n, const float2 *pv, float2 *t,
                      const KScalars *sc, cudaStream_t st) {
  const int g = (n + 255) / 256 < 2432 ? (n + 255) / 256 : 2432;
  launch_pdl(k_def_in_dd, g, 256, 0, st, n, c.azp, c.azj, c.azv_dd, c.y_dd, pv, t, sc);
  count_launches(1);
}

void launch_coarse_add_dd(const CoarseDev &c, float2 *z, const KScalars *sc,
                          cudaStream_t st) {
  k_coarse_add_dd<<<c.K, kCorrectBlock, 0, st>>>(c.sub_ptr, c.y_dd, z, sc);
  count_launches(1);
}

void launch_coarse_setup_b(const CoarseBatchDev &c, int K, int64_t n_blk,
                           const double *pvals, const int32_t *prp,
                           cudaStream_t st) {
  cudaMemsetAsync(c.ac, 0, (size_t)n_blk * sizeof(float), st);
  const size_t smem = (size_t)kCoarseBlock * c.max_cnb * sizeof(double);
  k_coarse_assemble_b<<<K, kCoarseBlock, smem, st>>>(c, prp, pvals);
  k_gj_block<<<c.n_sys, 1024, 3 * (size_t)c.max_k * sizeof(float), st>>>(c);
  count_launches(2);
}

void launch_coarse_apply_b(const CoarseBatchDev &c, int K, const double *in,
                           double *z, bool have_sums, const KScalars *sc,
                           cudaStream_t st) {
  if (!have_sums) {
    k_coarse_sum_b<<<K, kCoarseBlock, 0, st>>>(c, in, sc);
    count_launches(1);
  }
  k_coarse_correct_b<<<K, kCorrectBlock, 0, st>>>(c, z, sc);
  count_launches(1);
}

void launch_coarse_setup(const CoarseDev &c, const double *pvals,
                         const int32_t *prp, cudaGraphExec_t *gj_graph,
                         cudaStream_t st) {
  const int K = c.K;
  cudaMemsetAsync(c.ac, 0, (size_t)K * K * sizeof(float), st);
  const size_t smem = (size_t)kCoarseBlock * c.max_cnb * sizeof(double);
  k_coarse_assemble<<<K, kCoarseBlock, smem, st>>>(K, c.sub_ptr, prp, pvals,
                                                   c.cptr, c.cnb, c.cslot, c.ac);
  k_gj_diag<<<(K + 255) / 256, 256, 0, st>>>(K, c.ac, c.dg0);
  count_launches(2);
  // the K / kGjB block steps: captured once into a graph, replayed (run
  // directly when the capture is not possible)
  const int nblk = (K + kGjB - 1) / kGjB;
  const int nw = (K + 31) / 32;
  const dim3 ugrid((K + kUpdCols - 1) / kUpdCols, (K + kUpdRows - 1) / kUpdRows);
  // programmatic dependent launch: each kernel waits at entry for its
  // predecessor, so its launch overlaps the predecessor's tail
  auto steps = [&]() {
    for (int k0 = 0; k0 < K; k0 += kGjB) {
      const int b = K - k0 < kGjB ? K - k0 : kGjB;
      // the pivot inverse of step s is in pinv[s % 2] (the update of step
      // s - 1 writes it while step s - 1's own is still being read)
      float *pv = c.pinv + ((k0 / kGjB) & 1) * kGjB * kGjB;
      float *pv_next = c.pinv + (((k0 / kGjB) + 1) & 1) * kGjB * kGjB;
      launch_pdl(k_gjb_panel, nw + (4 * K + 255) / 256, 256, 0, st, K, k0, b,
                 nw, (const float *)c.ac, (const float *)c.dg0, pv,
                 k0 == 0 ? 1 : 0, c.W, c.V, c.C);
      // 16-byte rows need K % 4 == 0 (the buffer itself is 256-byte aligned)
      launch_pdl(K % 4 == 0 ? k_gjb_update<true> : k_gjb_update<false>, ugrid,
                 256, 0, st, K, k0, b, c.ac, (const float *)pv,
                 (const float *)c.dg0, pv_next, (const float *)c.W,
                 (const float *)c.V, (const float *)c.C);
    }
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
  count_launches(2 * nblk);
}

int launch_coarse_setup_lu(const CoarseDev &c, pg_lu *lu, double *cvals,
                           const double *pvals, const int32_t *prp,
                           cudaGraphExec_t *graph, cudaStream_t st) {
  // about 30 short dependent launches: captured once into a graph (per
  // inverse buffer), replayed; run directly when the capture fails
  int rc = PG_OK;
  auto run = [&]() {
    const size_t smem = (size_t)kCoarseBlock * c.max_cnb * sizeof(double);
    k_coarse_assemble_csr<<<c.K, kCoarseBlock, smem, st>>>(
        c.sub_ptr, prp, pvals, c.cptr, c.cslot, cvals);
    count_launches(1);
    return lu_inverse_run(lu, cvals, c.ac, st);
  };
  if (graph && !*graph) {
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed) == cudaSuccess) {
      rc = run();
      if (cudaStreamEndCapture(st, &g) == cudaSuccess && g && rc == PG_OK &&
          cudaGraphInstantiate(graph, g, 0) != cudaSuccess)
        *graph = nullptr;
      if (g) cudaGraphDestroy(g);
    }
    cudaGetLastError();  // a failed capture falls back to direct launches
  }
  if (graph && *graph) {
    // the capture counted the kernels of one run: a replay counts them
    // again only when it is not the capture's own first execution
    if (cudaGraphLaunch(*graph, st) != cudaSuccess) return run();
    if (lu_inverse_captured(lu)) count_launches(1 + lu_inverse_launches(lu));
    lu_inverse_set_captured(lu);
    return PG_OK;
  }
  return run();
}

void launch_coarse_apply(const CoarseDev &c, const double *in, double *z,
                         bool have_sums, const KScalars *sc, cudaStream_t st) {
  if (!have_sums) {
    k_coarse_sum<<<c.K, kCoarseBlock, 0, st>>>(c.sub_ptr, in, c.csum, sc);
    count_launches(1);
  }
  k_coarse_correct<double><<<c.K, kCorrectBlock, 0, st>>>(c.K, c.sub_ptr, c.ac,
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
  k_coarse_correct<float2><<<c.K, kCorrectBlock, 0, st>>>(c.K, c.sub_ptr, c.ac,
                                                          c.csum, z, sc);
  count_launches(1);
}

}  // namespace pg
