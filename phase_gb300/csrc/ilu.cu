// ILU(0) on Schwarz subdomains: numeric factorisation and the triangular
// sweeps, on the packed per-subdomain records described in kernels.cuh.
//
// Apply (the hot kernel): one warp owns one sweep group (one subdomain, or
// two independent ones whose levels share the warp's lanes).  Its factor is
// stored as a stream of level-aligned pieces (kernels.cuh StreamMeta); lane
// 0 moves the header and the first two pieces into shared memory with
// cp.async.bulk (TMA) while the warp stages the input vector, then refills
// the two alternating buffers (completed on mbarriers with bounded waits) so
// the next piece arrives while the current one is swept.  Within a piece the
// rows of a level are slot-major (the lanes read consecutive addresses); each
// lane reads its next level's columns and weights into registers while the
// current level is swept, and the warp synchronises with __syncwarp between
// levels.  A warp needs only header + 2 pieces + its z vector of shared
// memory (about 21 KB for 1024 FP64 rows), so several groups run per SM.
// With a coarse space the kernel also sums each subdomain's input.
#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "../../include/phase_gb300.h"
#include "dd.cuh"
#include "kernels.cuh"
#include "tma.cuh"

namespace pg {

namespace {

// Row-wise IKJ ILU(0) (Saad, Iterative Methods for Sparse Linear Systems,
// Alg. 10.4) on the diagonal block of one subdomain, in its record.  The CTA
// walks the level schedule; rows of one level depend only on rows of earlier
// levels, which the barrier has completed.  Pivots are FP64; the diagonal
// slot ends up holding 1/u_ii.
__global__ void k_ilu0_factor(const SubMeta *__restrict__ meta,
                              uint8_t *__restrict__ rec,
                              const int32_t *__restrict__ rec_src,
                              const double *__restrict__ pvals,
                              int *__restrict__ bad) {
  const SubMeta m = meta[blockIdx.x];
  uint8_t *base = rec + m.rec_off;
  const uint16_t *lvl = reinterpret_cast<const uint16_t *>(base);
  const uint16_t *cols = reinterpret_cast<const uint16_t *>(base + m.col_off);
  double *vals = reinterpret_cast<double *>(base + m.val_off);
  const int K = m.K, KL = m.KL, KU = K - KL, nr = m.nr;
  const int n_slots = nr * (K + 1);
  for (int j = threadIdx.x; j < n_slots; j += blockDim.x) {
    const int src = rec_src[m.slot_base + j];
    vals[j] = src >= 0 ? pvals[src] : 0.;
  }
  __syncthreads();
  double *dg = vals + (size_t)K * nr;
  for (int lv = 0; lv < m.nlev; ++lv) {
    const int a = lvl[lv], b = lvl[lv + 1];
    for (int i = a + threadIdx.x; i < b; i += blockDim.x) {
      for (int k = 0; k < KL; ++k) {
        const int c = cols[(size_t)k * nr + i];
        if (c == kPadCol) break;
        const double lik = vals[(size_t)k * nr + i] / dg[c];
        vals[(size_t)k * nr + i] = lik;
        // a_ij -= l_ik u_kj for the columns j of U(k) present in row i
        for (int q = 0; q < KU; ++q) {
          const int cu = cols[(size_t)(KL + q) * nr + c];
          if (cu == kPadCol) break;
          const double d = lik * vals[(size_t)(KL + q) * nr + c];
          if (cu == i) {
            dg[i] -= d;
            continue;
          }
          for (int k2 = 0; k2 < K; ++k2)
            if (cols[(size_t)k2 * nr + i] == cu) {
              vals[(size_t)k2 * nr + i] -= d;
              break;
            }
        }
      }
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < nr; i += blockDim.x) {
    const double piv = dg[i];
    if (piv == 0. || !isfinite(piv)) {
      atomicAdd(bad, 1);
      dg[i] = 0.;
    } else {
      dg[i] = 1. / piv;
    }
  }
}

// One level of a sweep: rows a .. a+w-1, slot-major columns cc and values vv
// (KS slots, compile-time when KT > 0), optional 1/u_ii dd.
template <class VT, class MT, int KT>
__device__ __forceinline__ void sweep_level(VT *zs, int a, int w, int ks,
                                            const uint16_t *cc, const MT *vv,
                                            const MT *dd, int lane) {
  const int K = KT > 0 ? KT : ks;
  for (int t = lane; t < w; t += 32) {
    VT acc = zs[a + t];
    if (KT > 0) {
#pragma unroll
      for (int k = 0; k < (KT > 0 ? KT : 1); ++k)
        acc -= (VT)vv[k * w + t] * zs[cc[k * w + t]];
    } else {
      for (int k = 0; k < K; ++k) acc -= (VT)vv[k * w + t] * zs[cc[k * w + t]];
    }
    zs[a + t] = dd ? acc * (VT)dd[t] : acc;
  }
}

// One level of a sweep in float-float arithmetic (dd.cuh): the products
// are accumulated with the compensated Dot2 scheme, so the level's serial
// dependence is one FP32 add per entry.
template <int KT>
__device__ __forceinline__ void sweep_level_dd(float2 *zs, int a, int w,
                                               int ks, const uint16_t *cc,
                                               const float2 *vv,
                                               const float2 *dd, int lane) {
  const int K = KT > 0 ? KT : ks;
  for (int t = lane; t < w; t += 32) {
    DdAcc acc = dd_acc(zs[a + t]);
    if (KT > 0) {
#pragma unroll
      for (int k = 0; k < (KT > 0 ? KT : 1); ++k)
        dd_acc_fma(acc, dd_neg(vv[k * w + t]), zs[cc[k * w + t]]);
    } else {
      for (int k = 0; k < K; ++k)
        dd_acc_fma(acc, dd_neg(vv[k * w + t]), zs[cc[k * w + t]]);
    }
    const float2 out = dd_value(acc);
    zs[a + t] = dd ? dd_mul(out, dd[t]) : out;
  }
}

// A level of a sweep group: rows [a0, a0+w0) of its first subdomain and
// [a1, a1+w1) of its second (group-local); lane t sweeps row(t)
struct GroupLevel {
  int a0 = 0, w0 = 0, a1 = 0, w1 = 0;
  __device__ __forceinline__ int w() const { return w0 + w1; }
  __device__ __forceinline__ int row(int t) const {
    return t < w0 ? a0 + t : a1 + (t - w0);
  }
};
__device__ __forceinline__ GroupLevel group_level(const uint2 *L, int l) {
  const uint2 x = L[l];
  GroupLevel g;
  g.a0 = (int)(x.x & 0xFFFFu);
  g.w0 = (int)(x.x >> 16);
  g.a1 = (int)(x.y & 0xFFFFu);
  g.w1 = (int)(x.y >> 16);
  return g;
}

// One lane's row of a level (lane < w), held in registers: the KT column
// slots, their weights and, for the backward sweep, 1/u_ii.  Record layout
// of a level of width w: columns (uint16, slot-major, 16-byte padded), the
// weights (slot-major, padded), then 1/u_ii for a backward level.
template <class V, int KT>
struct LevelRegs {
  uint16_t c[KT];
  V v[KT];
  V d;
  template <bool DIAG>
  __device__ __forceinline__ void load(const uint8_t *p, int w, int lane) {
    if (lane >= w || w > 32) return;
    const uint16_t *cp = reinterpret_cast<const uint16_t *>(p);
    const V *vp = reinterpret_cast<const V *>(p + al16(2 * KT * w));
#pragma unroll
    for (int k = 0; k < KT; ++k) {
      c[k] = cp[k * w + lane];
      v[k] = vp[k * w + lane];
    }
    if (DIAG)
      d = reinterpret_cast<const V *>(p + al16(2 * KT * w) +
                                      al16((int)sizeof(V) * KT * w))[lane];
  }
  // the row's new z: (z_self - sum_k v_k z[c_k]) (* 1/u_ii), with the
  // arithmetic of sweep_level / sweep_level_dd
  template <class AR, bool DIAG>
  __device__ __forceinline__ V sweep(const V *zs, V self) const {
    V x[KT];
#pragma unroll
    for (int k = 0; k < KT; ++k) x[k] = zs[c[k]];
    return AR::template row<KT, DIAG>(self, v, x, d);
  }
};

// Arithmetic of the streamed sweep: FP64, or float-float on the same
// record layout (a float pair takes the 8 bytes of a double).
struct ArithF64 {
  using V = double;
  __device__ static V pre(int mode, int i, const V *r, V *pv, const V *v,
                          const KScalars *sc) {
    return pre_input<double>(mode, i, r, pv, v, sc);
  }
  __device__ static V combine(int mode, V ri, V pi, V vi, const KScalars *sc) {
    return pre_combine<double>(mode, ri, pi, vi, sc);
  }
  __device__ static V zero() { return 0.; }
  // output z + y_s of the deflated form (mode 3)
  __device__ static V add_y(V z, const void *y, int sub) {
    return z + static_cast<const double *>(y)[sub];
  }
  __device__ static V load_y(const void *y, int sub) {
    return static_cast<const double *>(y)[sub];
  }
  __device__ static V add(V a, V b) { return a + b; }
  // subdomain sums for the coarse correction
  using Sum = double;
  __device__ static Sum sum_init() { return 0.; }
  __device__ static void sum_add(Sum &a, V x) { a += x; }
  __device__ static float2 sum_warp(Sum a) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    return dd_from(a);
  }
  template <int KT, bool DIAG>
  __device__ static V row(V self, const V (&v)[KT], const V (&x)[KT], V d) {
    V acc = self;
#pragma unroll
    for (int k = 0; k < KT; ++k) acc -= v[k] * x[k];
    return DIAG ? acc * d : acc;
  }
  template <int KT>
  __device__ static void level(V *zs, int a, int w, int ks,
                               const uint16_t *cc, const V *vv, const V *dd,
                               int lane) {
    sweep_level<double, double, KT>(zs, a, w, ks, cc, vv, dd, lane);
  }
};
struct ArithDD {
  using V = float2;
  __device__ static V pre(int mode, int i, const V *r, V *pv, const V *v,
                          const KScalars *sc) {
    return dd_pre_input(mode, i, r, pv, v, sc);
  }
  __device__ static V combine(int mode, V ri, V pi, V vi, const KScalars *sc) {
    return dd_pre_combine(mode, ri, pi, vi, sc);
  }
  __device__ static V zero() { return make_float2(0.f, 0.f); }
  __device__ static V add_y(V z, const void *y, int sub) {
    return dd_add(z, static_cast<const float2 *>(y)[sub]);
  }
  __device__ static V load_y(const void *y, int sub) {
    return static_cast<const float2 *>(y)[sub];
  }
  __device__ static V add(V a, V b) { return dd_add(a, b); }
  using Sum = DdAcc;
  __device__ static Sum sum_init() { return dd_acc(make_float2(0.f, 0.f)); }
  __device__ static void sum_add(Sum &a, V x) { dd_acc_add(a, x); }
  __device__ static float2 sum_warp(Sum a) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      DdAcc b;
      b.s = __shfl_xor_sync(0xffffffffu, a.s, o);
      b.c = __shfl_xor_sync(0xffffffffu, a.c, o);
      dd_acc_merge(a, b);
    }
    return dd_value(a);
  }
  template <int KT, bool DIAG>
  __device__ static V row(V self, const V (&v)[KT], const V (&x)[KT], V d) {
    DdAcc acc = dd_acc(self);
#pragma unroll
    for (int k = 0; k < KT; ++k) dd_acc_fma(acc, dd_neg(v[k]), x[k]);
    const float2 out = dd_value(acc);
    return DIAG ? dd_mul(out, d) : out;
  }
  template <int KT>
  __device__ static void level(V *zs, int a, int w, int ks,
                               const uint16_t *cc, const V *vv, const V *dd,
                               int lane) {
    sweep_level_dd<KT>(zs, a, w, ks, cc, vv, dd, lane);
  }
};

// Forward/backward sweeps of one subdomain by one warp (see file header).
// Shared memory: header | piece buffer 0 | piece buffer 1 | z[nr+1].  Piece
// j+2 is loaded into the buffer piece j used while piece j+1 is being
// swept.  KLT/KUT fix the L/U slot counts at compile time (0 = from meta).
template <class AR, int MODE, int KLT, int KUT>
__global__ void __launch_bounds__(32)
k_ilu0_apply_stream(const StreamMeta *__restrict__ meta,
                    const uint8_t *__restrict__ rec,
                    const typename AR::V *__restrict__ r,
                    typename AR::V *__restrict__ pv,
                    const typename AR::V *__restrict__ v,
                    typename AR::V *__restrict__ z,
                    const KScalars *__restrict__ sc_base,
                    const int32_t *__restrict__ sub_sys,
                    int *__restrict__ err, float2 *__restrict__ csum,
                    const void *__restrict__ def_y) {
  using MT = typename AR::V;
  // batched solves: the scalars of this subdomain's system
  const KScalars *sc =
      sc_base && sub_sys ? sc_base + sub_sys[blockIdx.x] : sc_base;
  pdl_wait();
  if (sc && sc->done) return;
  extern __shared__ __align__(128) uint8_t smem[];
  __shared__ __align__(8) uint64_t bar[3];
  const StreamMeta m = meta[blockIdx.x];
  const int lane = threadIdx.x;
  const int nr = m.nr, nlev = m.nlev;
  const int KL = KLT > 0 ? KLT : m.KL, KU = KUT > 0 ? KUT : m.KU;
  uint8_t *hdr = smem;
  uint8_t *const buf0 = smem + m.hdr_bytes;  // buffer b at buf0 + b*max_piece
  MT *zs = reinterpret_cast<MT *>(smem + m.hdr_bytes + 2 * m.max_piece);
  const uint8_t *g = rec + m.rec_off;
  // the header and the first two pieces are in flight while the input is
  // staged
  if (lane == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_init(&bar[2], 1);
    mbar_expect_tx(&bar[2], (uint32_t)m.hdr_bytes);
    bulk_load(hdr, g, (uint32_t)m.hdr_bytes, &bar[2]);
    mbar_expect_tx(&bar[0], (uint32_t)m.p0_bytes);
    bulk_load(buf0, g + m.p0_off, (uint32_t)m.p0_bytes, &bar[0]);
    if (m.p1_bytes > 0) {
      mbar_expect_tx(&bar[1], (uint32_t)m.p1_bytes);
      bulk_load(buf0 + m.max_piece, g + m.p1_off, (uint32_t)m.p1_bytes,
                &bar[1]);
    }
  }
  {
    // input staging, four rows per lane in flight; with a coarse space the
    // input sum of each subdomain of the group (lane order, then a fixed
    // butterfly)
    constexpr int U = 4;
    const MT zero = AR::zero();
    typename AR::Sum part0 = AR::sum_init(), part1 = AR::sum_init();
    for (int i0 = lane; i0 < nr; i0 += 32 * U) {
      MT ri[U], pi[U], vi[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int i = i0 + 32 * u;
        ri[u] = pi[u] = vi[u] = zero;
        if (i < nr) {
          if (MODE == 1 || MODE == 2) ri[u] = r[m.r0 + i], vi[u] = v[m.r0 + i];
          if (MODE != 2) pi[u] = pv[m.r0 + i];
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int i = i0 + 32 * u;
        if (i < nr) {
          MT val;
          if constexpr (MODE == 3)
            val = pi[u];
          else
            val = AR::combine(MODE, ri[u], pi[u], vi[u], sc);
          if (MODE == 1 || MODE == 2) pv[m.r0 + i] = val;
          zs[i] = val;
          if (csum) AR::sum_add(i < m.nr0 ? part0 : part1, val);
        }
      }
    }
    if (csum) {
      const float2 t0 = AR::sum_warp(part0);
      if (lane == 0) csum[m.sub0] = t0;
      if (m.nsub > 1) {
        const float2 t1 = AR::sum_warp(part1);
        if (lane == 0) csum[m.sub0 + 1] = t1;
      }
    }
  }
  if (lane == 0) zs[nr] = AR::zero();
  __syncwarp();
  if (!mbar_wait_bounded(&bar[2], err)) {
    // the first pieces are in flight: wait for them (bounded), leave
    mbar_wait_bounded(&bar[0], nullptr, 0u);
    if (m.p1_bytes > 0) mbar_wait_bounded(&bar[1], nullptr, 0u);
    return;
  }
  const uint2 *L = reinterpret_cast<const uint2 *>(hdr);  // lev[nlev][4]
  const int32_t *ints = reinterpret_cast<const int32_t *>(hdr + 8 * nlev);
  const int nF = ints[0], nB = ints[1], P = nF + nB;
  const int32_t *tab = ints + 2;
  constexpr int vs = (int)sizeof(MT);
  uint32_t phases = 0u;  // bit b: parity to wait for on buffer b
  for (int j = 0; j < P; ++j) {
    const int sb = j & 1;
    if (!mbar_wait_bounded(&bar[sb], err, (phases >> sb) & 1u)) {
      // a load in flight in the other buffer: wait for it (bounded), leave
      if (j + 1 < P)
        mbar_wait_bounded(&bar[sb ^ 1], nullptr, (phases >> (sb ^ 1)) & 1u);
      return;
    }
    phases ^= 1u << sb;
    const uint8_t *pc = buf0 + sb * m.max_piece;
    if constexpr (KLT > 0 && KUT > 0) {
      // Software-pipelined walk: a level's columns, weights (and 1/u_ii)
      // are read from the piece into registers while the level before it
      // is swept, so each level waits only for its z operands.  Levels
      // wider than a warp (single-subdomain groups only) take the generic
      // loop.
      if (j < nF) {
        const int l0 = tab[3 * j];
        const int l1 = j + 1 < nF ? tab[3 * (j + 1)] : nlev;
        GroupLevel cl = group_level(L, l0);
        int w = cl.w();
        LevelRegs<MT, KLT> cur, nxt;
        cur.template load<false>(pc, w, lane);
        for (int l = l0; l < l1; ++l) {
          const int ca = al16(2 * KLT * w);
          const uint8_t *pn = pc + ca + al16(vs * KLT * w);
          const GroupLevel nl = l + 1 < l1 ? group_level(L, l + 1) : GroupLevel{};
          const int wn = nl.w();
          nxt.template load<false>(pn, wn, lane);
          if (w <= 32) {
            if (lane < w) {
              const int row = cl.row(lane);
              zs[row] = cur.template sweep<AR, false>(zs, zs[row]);
            }
          } else {
            AR::template level<KLT>(zs, cl.a0, cl.w0, KLT,
                                     reinterpret_cast<const uint16_t *>(pc),
                                     reinterpret_cast<const MT *>(pc + ca),
                                     (const MT *)nullptr, lane);
          }
          cl = nl;
          w = wn;
          pc = pn;
          cur = nxt;
          __syncwarp();
        }
      } else {
        const int lhi = tab[3 * j];
        const int llo = j + 1 < P ? tab[3 * (j + 1)] + 1 : 0;
        GroupLevel cl = group_level(L, lhi);
        int w = cl.w();
        LevelRegs<MT, KUT> cur, nxt;
        cur.template load<true>(pc, w, lane);
        for (int l = lhi; l >= llo; --l) {
          const int ca = al16(2 * KUT * w), va = al16(vs * KUT * w);
          const uint8_t *pn = pc + ca + va + al16(vs * w);
          const GroupLevel nl = l - 1 >= llo ? group_level(L, l - 1) : GroupLevel{};
          const int wn = nl.w();
          nxt.template load<true>(pn, wn, lane);
          if (w <= 32) {
            if (lane < w) {
              const int row = cl.row(lane);
              zs[row] = cur.template sweep<AR, true>(zs, zs[row]);
            }
          } else {
            AR::template level<KUT>(zs, cl.a0, cl.w0, KUT,
                                     reinterpret_cast<const uint16_t *>(pc),
                                     reinterpret_cast<const MT *>(pc + ca),
                                     reinterpret_cast<const MT *>(pc + ca + va),
                                     lane);
          }
          cl = nl;
          w = wn;
          pc = pn;
          cur = nxt;
          __syncwarp();
        }
      }
    } else if (j < nF) {
      // generic slot counts: single-subdomain groups (w1 = 0)
      const int l1 = j + 1 < nF ? tab[3 * (j + 1)] : nlev;
      for (int l = tab[3 * j]; l < l1; ++l) {
        const GroupLevel cl = group_level(L, l);
        const int a = cl.a0, w = cl.w0;
        const int ca = al16(2 * KL * w);
        AR::template level<KLT>(zs, a, w, KL,
                                 reinterpret_cast<const uint16_t *>(pc),
                                 reinterpret_cast<const MT *>(pc + ca),
                                 (const MT *)nullptr, lane);
        pc += ca + al16(vs * KL * w);
        __syncwarp();
      }
    } else {
      const int lhi = tab[3 * j];
      const int llo = j + 1 < P ? tab[3 * (j + 1)] + 1 : 0;
      for (int l = lhi; l >= llo; --l) {
        const GroupLevel cl = group_level(L, l);
        const int a = cl.a0, w = cl.w0;
        const int ca = al16(2 * KU * w), va = al16(vs * KU * w);
        AR::template level<KUT>(zs, a, w, KU,
                                 reinterpret_cast<const uint16_t *>(pc),
                                 reinterpret_cast<const MT *>(pc + ca),
                                 reinterpret_cast<const MT *>(pc + ca + va),
                                 lane);
        pc += ca + va + al16(vs * w);
        __syncwarp();
      }
    }
    if (lane == 0 && j + 2 < P) {
      // the generic-proxy reads of this buffer are ordered before the
      // async-proxy refill
      fence_proxy_async();
      mbar_expect_tx(&bar[sb], (uint32_t)tab[3 * (j + 2) + 2]);
      bulk_load(buf0 + sb * m.max_piece, g + tab[3 * (j + 2) + 1],
                (uint32_t)tab[3 * (j + 2) + 2], &bar[sb]);
    }
  }
  if constexpr (MODE == 3) {
    const MT y0 = AR::load_y(def_y, m.sub0);
    const MT y1 = m.nsub > 1 ? AR::load_y(def_y, m.sub0 + 1) : y0;
    for (int i = lane; i < nr; i += 32)
      z[m.r0 + i] = AR::add(zs[i], i < m.nr0 ? y0 : y1);
  } else {
    for (int i = lane; i < nr; i += 32) z[m.r0 + i] = zs[i];
  }
}

// Line-form sweeps (kernels.cuh LineMeta) of a group of structured blocks.
// Lane i of a member walks grid line i, one row per level: on level l it
// owns position s = l - i of its line.  Forward, z(i, j) = x(i, j) - f0
// z(i-1, j) - f1 z(i, j-1): z(i-1, j) is lane i-1's result of level l-1 (a
// shuffle) and z(i, j-1) the lane's own (`carry`); backward, z(i, j) =
// (z(i, j) - b1 z(i, j+1) - b0 z(i+1, j)) / u_ii with z(i+1, j) from lane
// i+1.  The group's vector is copied into line-major order in shared memory
// and the weights are stored line by line, so a lane's next row and
// weights are consecutive and read one level ahead; the chain of a level is
// a shuffle and two multiply-adds.  The products are subtracted in the
// order of the row's factor slots (increasing column), as the stream form
// does, so both give the same results.  The record's map and both weight
// arrays are bulk-copied into shared memory at kernel start; the input is
// staged through the map with the subdomain sums taken in the stream
// form's order, and the output (with y_s in mode 3) goes back through it.
template <class AR>
__device__ __forceinline__ typename AR::V shfl_up_v(typename AR::V x, int w);
template <>
__device__ __forceinline__ double shfl_up_v<ArithF64>(double x, int w) {
  return __shfl_up_sync(0xffffffffu, x, 1, w);
}
template <>
__device__ __forceinline__ float2 shfl_up_v<ArithDD>(float2 x, int w) {
  return make_float2(__shfl_up_sync(0xffffffffu, x.x, 1, w),
                     __shfl_up_sync(0xffffffffu, x.y, 1, w));
}
template <class AR>
__device__ __forceinline__ typename AR::V shfl_down_v(typename AR::V x, int w);
template <>
__device__ __forceinline__ double shfl_down_v<ArithF64>(double x, int w) {
  return __shfl_down_sync(0xffffffffu, x, 1, w);
}
template <>
__device__ __forceinline__ float2 shfl_down_v<ArithDD>(float2 x, int w) {
  return make_float2(__shfl_down_sync(0xffffffffu, x.x, 1, w),
                     __shfl_down_sync(0xffffffffu, x.y, 1, w));
}

// One row of a line sweep: self - w0 x0 - w1 x1 (* d), with the weights in
// their storage type WT (the vector arithmetic's own type, or FP32 weights
// in float-float arithmetic).
template <class AR, class WT, bool DIAG>
__device__ __forceinline__ typename AR::V line_row(typename AR::V self, WT w0,
                                                   WT w1, typename AR::V x0,
                                                   typename AR::V x1, WT d) {
  if constexpr (std::is_same<WT, float>::value) {
    DdAcc acc = dd_acc(self);
    dd_acc_fma_f(acc, -w0, x0);
    dd_acc_fma_f(acc, -w1, x1);
    const float2 out = dd_value(acc);
    return DIAG ? dd_mul_f(out, d) : out;
  } else {
    const typename AR::V wv[2] = {w0, w1}, zv[2] = {x0, x1};
    return AR::template row<2, DIAG>(self, wv, zv, d);
  }
}

template <class AR, int MODE, class WT>
__global__ void __launch_bounds__(32)
k_ilu0_apply_line(const LineMeta *__restrict__ meta,
                  const uint8_t *__restrict__ rec,
                  const typename AR::V *__restrict__ r,
                  typename AR::V *__restrict__ pv,
                  const typename AR::V *__restrict__ v,
                  typename AR::V *__restrict__ z,
                  const KScalars *__restrict__ sc, int *__restrict__ err,
                  float2 *__restrict__ csum, const void *__restrict__ def_y) {
  using MT = typename AR::V;
  pdl_wait();
  if (sc && sc->done) return;
  extern __shared__ __align__(128) uint8_t smem[];
  __shared__ __align__(8) uint64_t bar[3];
  const LineMeta m = meta[blockIdx.x];
  const int lane = threadIdx.x;
  const int nr = m.nr, nlev = m.nlev;
  uint8_t *hdr = smem;
  uint8_t *const buf0 = smem + m.hdr_bytes;
  // the group's vector, in line-major order
  MT *zl = reinterpret_cast<MT *>(smem + m.zs_off);
  const uint8_t *g = rec + m.rec_off;
  // used for FP32 weights only (the map and both weight arrays fit in
  // shared memory beside the group's vector); 8-byte weights take the
  // level-major form, k_ilu0_apply_line_lv
  constexpr bool kSmemW = true;
  if (lane == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_init(&bar[2], 1);
    mbar_expect_tx(&bar[2], (uint32_t)m.hdr_bytes);
    bulk_load(hdr, g, (uint32_t)m.hdr_bytes, &bar[2]);
    if (kSmemW) {
      mbar_expect_tx(&bar[0], (uint32_t)m.p0_bytes);
      bulk_load(buf0, g + m.p0_off, (uint32_t)m.p0_bytes, &bar[0]);
      mbar_expect_tx(&bar[1], (uint32_t)m.p1_bytes);
      bulk_load(buf0 + m.buf1, g + m.p1_off, (uint32_t)m.p1_bytes, &bar[1]);
    }
  }
  __syncwarp();  // lane 0 has initialised the barriers
  // the level-order -> line-major map, then the input staged through it
  // (the subdomain sums in lane-strided level order)
  if (!mbar_wait_bounded(&bar[2], err)) {
    if (kSmemW) {
      mbar_wait_bounded(&bar[0], nullptr, 0u);
      mbar_wait_bounded(&bar[1], nullptr, 0u);
    }
    return;
  }
  const uint16_t *map = reinterpret_cast<const uint16_t *>(hdr);
  {
    constexpr int U = 4;
    const MT zero = AR::zero();
    typename AR::Sum part0 = AR::sum_init(), part1 = AR::sum_init();
    for (int i0 = lane; i0 < nr; i0 += 32 * U) {
      MT ri[U], pi[U], vi[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int i = i0 + 32 * u;
        ri[u] = pi[u] = vi[u] = zero;
        if (i < nr) {
          if (MODE == 1 || MODE == 2) ri[u] = r[m.r0 + i], vi[u] = v[m.r0 + i];
          if (MODE != 2) pi[u] = pv[m.r0 + i];
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int i = i0 + 32 * u;
        if (i < nr) {
          MT val;
          if constexpr (MODE == 0 || MODE == 3)
            val = pi[u];
          else
            val = AR::combine(MODE, ri[u], pi[u], vi[u], sc);
          if (MODE == 1 || MODE == 2) pv[m.r0 + i] = val;
          zl[map[i]] = val;
          if (csum) AR::sum_add(i < m.nr0 ? part0 : part1, val);
        }
      }
    }
    if (csum) {
      const float2 t0 = AR::sum_warp(part0);
      if (lane == 0) csum[m.sub0] = t0;
      if (m.nsub > 1) {
        const float2 t1 = AR::sum_warp(part1);
        if (lane == 0) csum[m.sub0 + 1] = t1;
      }
    }
  }
  const int width = m.lanes;  // shuffle segment: 16 (pair) or 32
  const int mem = width == 16 ? lane >> 4 : 0;
  const int li = width == 16 ? lane & 15 : lane;
  const int len = mem ? m.len1 : m.len0;
  const bool mine = li < (mem ? m.lines1 : m.lines0);
  const int pos0 = (mem ? m.nr0 : 0) + li * len;  // this lane's line start
  MT *zline = zl + pos0;
  __syncwarp();
  // forward: on level l this lane owns position s = l - li of its line;
  // weights are read two positions ahead, the row one position ahead
  if (kSmemW && !mbar_wait_bounded(&bar[0], err, 0u)) {
    mbar_wait_bounded(&bar[1], nullptr, 0u);
    return;
  }
  {
    const WT *fw = reinterpret_cast<const WT *>(kSmemW ? buf0 : g + m.p0_off) +
                   2 * pos0;
    MT carry = AR::zero();
    WT f0 = WT(), f1 = WT(), g0 = WT(), g1 = WT();
    MT x = AR::zero();
    if (mine && len > 0) {
      f0 = fw[0];
      f1 = fw[1];
      x = zline[0];
      if (len > 1) {
        g0 = fw[2];
        g1 = fw[3];
      }
    }
#pragma unroll 2
    for (int l = 0; l < nlev; ++l) {
      const int sp = l - li;
      const bool ok = mine && (unsigned)sp < (unsigned)len;
      WT h0 = g0, h1 = g1;
      MT xn = x;
      if (ok && sp + 2 < len) {
        h0 = fw[2 * (sp + 2)];
        h1 = fw[2 * (sp + 2) + 1];
      }
      if (ok && sp + 1 < len) xn = zline[sp + 1];
      MT left = shfl_up_v<AR>(carry, width);
      if (li == 0) left = AR::zero();
      MT out = AR::zero();
      if (ok) {
        out = line_row<AR, WT, false>(x, f0, f1, left, carry, WT());
        zline[sp] = out;
        f0 = g0;
        f1 = g1;
        g0 = h0;
        g1 = h1;
        x = xn;
      }
      carry = out;
    }
  }
  // backward: on level l this lane owns position s = l - li, descending
  if (kSmemW && !mbar_wait_bounded(&bar[1], err, 0u)) return;
  {
    const WT *bw = reinterpret_cast<const WT *>(kSmemW ? buf0 + m.buf1
                                                       : g + m.p1_off) +
                   3 * pos0;
    MT carry = AR::zero();
    WT b0 = WT(), b1 = WT(), dg = WT(), c0 = WT(), c1 = WT(), cd = WT();
    MT x = AR::zero();
    const int last = len - 1;
    if (mine && len > 0) {
      b0 = bw[3 * last];
      b1 = bw[3 * last + 1];
      dg = bw[3 * last + 2];
      x = zline[last];
      if (last > 0) {
        c0 = bw[3 * (last - 1)];
        c1 = bw[3 * (last - 1) + 1];
        cd = bw[3 * (last - 1) + 2];
      }
    }
#pragma unroll 2
    for (int l = nlev - 1; l >= 0; --l) {
      const int sp = l - li;
      const bool ok = mine && (unsigned)sp < (unsigned)len;
      WT e0 = c0, e1 = c1, ed = cd;
      MT xn = x;
      if (ok && sp > 1) {
        e0 = bw[3 * (sp - 2)];
        e1 = bw[3 * (sp - 2) + 1];
        ed = bw[3 * (sp - 2) + 2];
      }
      if (ok && sp > 0) xn = zline[sp - 1];
      MT right = shfl_down_v<AR>(carry, width);
      if (li == width - 1) right = AR::zero();
      MT out = AR::zero();
      if (ok) {
        // U slots in increasing column: (i, j+1) (this lane's line) is on
        // an earlier line than (i+1, j)
        out = line_row<AR, WT, true>(x, b1, b0, carry, right, dg);
        zline[sp] = out;
        b0 = c0;
        b1 = c1;
        dg = cd;
        c0 = e0;
        c1 = e1;
        cd = ed;
        x = xn;
      }
      carry = out;
    }
  }
  __syncwarp();
  if constexpr (MODE == 3) {
    // y of the group's (at most two) subdomains, read once
    const MT y0 = AR::load_y(def_y, m.sub0);
    const MT y1 = m.nsub > 1 ? AR::load_y(def_y, m.sub0 + 1) : y0;
    for (int i = lane; i < nr; i += 32)
      z[m.r0 + i] = AR::add(zl[map[i]], i < m.nr0 ? y0 : y1);
  } else {
    for (int i = lane; i < nr; i += 32) z[m.r0 + i] = zl[map[i]];
  }
}

// a level's members: start row, rows, first line
struct LineLevel {
  int a, w, lo, t0;  // this lane's member: rows a .. a+w-1 on lines lo ..;
                     // its entries start at t0 in the level blob
  int wsum;          // entries of the level (both members)
};
__device__ __forceinline__ LineLevel line_level(const uint2 *L, int l,
                                                int mem) {
  const uint2 x = L[l];
  const int w0 = (int)(x.y & 0xFFu), w1 = (int)((x.y >> 16) & 0xFFu);
  LineLevel g;
  g.a = mem ? (int)(x.x >> 16) : (int)(x.x & 0xFFFFu);
  g.w = mem ? w1 : w0;
  g.lo = mem ? (int)(x.y >> 24) : (int)((x.y >> 8) & 0xFFu);
  g.t0 = mem ? w0 : 0;
  g.wsum = w0 + w1;
  return g;
}

// Level-major form of the line sweep, for 8-byte weights (FP64 records and
// their float-pair copies): the record is a header of per-level member
// tables and level blobs of weights (kernels.cuh LineMeta, built by
// analyse() for these records), streamed through two shared-memory buffers
// by TMA, so a group needs little shared memory; lane i's entry of level l
// is found from the level's table.  Same arithmetic, in the same order, as
// k_ilu0_apply_line.
template <class AR, int MODE, class WT>
__global__ void __launch_bounds__(32)
k_ilu0_apply_line_lv(const LineMeta *__restrict__ meta,
                  const uint8_t *__restrict__ rec,
                  const typename AR::V *__restrict__ r,
                  typename AR::V *__restrict__ pv,
                  const typename AR::V *__restrict__ v,
                  typename AR::V *__restrict__ z,
                  const KScalars *__restrict__ sc, int *__restrict__ err,
                  float2 *__restrict__ csum, const void *__restrict__ def_y) {
  using MT = typename AR::V;
  pdl_wait();
  if (sc && sc->done) return;
  extern __shared__ __align__(128) uint8_t smem[];
  __shared__ __align__(8) uint64_t bar[4];
  const LineMeta m = meta[blockIdx.x];
  const int lane = threadIdx.x;
  const int nr = m.nr, nlev = m.nlev;
  uint8_t *hdr = smem;
  uint8_t *const buf0 = smem + m.hdr_bytes;
  MT *zs = reinterpret_cast<MT *>(smem + m.zs_off);
  const uint8_t *g = rec + m.rec_off;
  // modes 0 and 3 read one input vector: one bulk copy straight into z,
  // in flight with the factor pieces (16-byte aligned ranges only)
  const bool tma_in =
      (MODE == 0 || MODE == 3) && (nr & 1) == 0 &&
      (reinterpret_cast<uintptr_t>(pv + m.r0) & 15u) == 0;
  if (lane == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    mbar_init(&bar[2], 1);
    mbar_init(&bar[3], 1);
    mbar_expect_tx(&bar[2], (uint32_t)m.hdr_bytes);
    bulk_load(hdr, g, (uint32_t)m.hdr_bytes, &bar[2]);
    if (tma_in) {
      mbar_expect_tx(&bar[3], (uint32_t)(nr * sizeof(MT)));
      bulk_load(zs, pv + m.r0, (uint32_t)(nr * sizeof(MT)), &bar[3]);
    }
    mbar_expect_tx(&bar[0], (uint32_t)m.p0_bytes);
    bulk_load(buf0, g + m.p0_off, (uint32_t)m.p0_bytes, &bar[0]);
    if (m.p1_bytes > 0) {
      mbar_expect_tx(&bar[1], (uint32_t)m.p1_bytes);
      bulk_load(buf0 + m.buf1, g + m.p1_off, (uint32_t)m.p1_bytes, &bar[1]);
    }
  }
  if (tma_in) {
    __syncwarp();  // lane 0 has initialised the barriers
    if (!mbar_wait_bounded(&bar[3], err)) {
      mbar_wait_bounded(&bar[2], nullptr, 0u);
      mbar_wait_bounded(&bar[0], nullptr, 0u);
      if (m.p1_bytes > 0) mbar_wait_bounded(&bar[1], nullptr, 0u);
      return;
    }
    if (csum) {  // the same lane-strided order as the register staging
      typename AR::Sum part0 = AR::sum_init(), part1 = AR::sum_init();
      for (int i = lane; i < nr; i += 32)
        AR::sum_add(i < m.nr0 ? part0 : part1, zs[i]);
      const float2 t0 = AR::sum_warp(part0);
      if (lane == 0) csum[m.sub0] = t0;
      if (m.nsub > 1) {
        const float2 t1 = AR::sum_warp(part1);
        if (lane == 0) csum[m.sub0 + 1] = t1;
      }
    }
  } else {
    constexpr int U = 4;
    const MT zero = AR::zero();
    typename AR::Sum part0 = AR::sum_init(), part1 = AR::sum_init();
    for (int i0 = lane; i0 < nr; i0 += 32 * U) {
      MT ri[U], pi[U], vi[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int i = i0 + 32 * u;
        ri[u] = pi[u] = vi[u] = zero;
        if (i < nr) {
          if (MODE == 1 || MODE == 2) ri[u] = r[m.r0 + i], vi[u] = v[m.r0 + i];
          if (MODE != 2) pi[u] = pv[m.r0 + i];
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const int i = i0 + 32 * u;
        if (i < nr) {
          MT val;
          if constexpr (MODE == 3)
            val = pi[u];
          else
            val = AR::combine(MODE, ri[u], pi[u], vi[u], sc);
          if (MODE == 1 || MODE == 2) pv[m.r0 + i] = val;
          zs[i] = val;
          if (csum) AR::sum_add(i < m.nr0 ? part0 : part1, val);
        }
      }
    }
    if (csum) {
      const float2 t0 = AR::sum_warp(part0);
      if (lane == 0) csum[m.sub0] = t0;
      if (m.nsub > 1) {
        const float2 t1 = AR::sum_warp(part1);
        if (lane == 0) csum[m.sub0 + 1] = t1;
      }
    }
  }
  __syncwarp();
  if (!mbar_wait_bounded(&bar[2], err)) {
    mbar_wait_bounded(&bar[0], nullptr, 0u);
    if (m.p1_bytes > 0) mbar_wait_bounded(&bar[1], nullptr, 0u);
    return;
  }
  const uint2 *L = reinterpret_cast<const uint2 *>(hdr);
  const int32_t *ints = reinterpret_cast<const int32_t *>(hdr + 8 * nlev);
  const int nF = ints[0], nB = ints[1], P = nF + nB;
  const int32_t *tab = ints + 2;
  constexpr int vs = (int)sizeof(WT);
  const int width = m.lanes;  // shuffle segment: 16 (pair) or 32
  const int mem = width == 16 ? lane >> 4 : 0;
  const int li = width == 16 ? lane & 15 : lane;
  MT carry = AR::zero();
  uint32_t phases = 0u;
  for (int j = 0; j < P; ++j) {
    const int sb = j & 1;
    if (!mbar_wait_bounded(&bar[sb], err, (phases >> sb) & 1u)) {
      if (j + 1 < P)
        mbar_wait_bounded(&bar[sb ^ 1], nullptr, (phases >> (sb ^ 1)) & 1u);
      return;
    }
    phases ^= 1u << sb;
    const uint8_t *pc = buf0 + (sb ? m.buf1 : 0);
    if (j == nF) carry = AR::zero();  // the backward sweep starts
    if (j < nF) {
      const int l0 = tab[3 * j];
      const int l1 = j + 1 < nF ? tab[3 * (j + 1)] : nlev;
      // operands of level l0, then each level reads the next one's
      LineLevel cl = line_level(L, l0, mem);
      int k = li - cl.lo;
      bool ok = (unsigned)k < (unsigned)cl.w;
      WT f0 = WT(), f1 = WT();
      MT x = AR::zero();
      if (ok) {
        const WT *fp = reinterpret_cast<const WT *>(pc) + 2 * (cl.t0 + k);
        f0 = fp[0];
        f1 = fp[1];
        x = zs[cl.a + k];
      }
      for (int l = l0; l < l1; ++l) {
        const uint8_t *pn = pc + al16(2 * vs * cl.wsum);
        LineLevel nl{};
        int kn = 0;
        bool okn = false;
        WT g0 = WT(), g1 = WT();
        MT xn = AR::zero();
        if (l + 1 < l1) {
          nl = line_level(L, l + 1, mem);
          kn = li - nl.lo;
          okn = (unsigned)kn < (unsigned)nl.w;
          if (okn) {
            const WT *fp = reinterpret_cast<const WT *>(pn) + 2 * (nl.t0 + kn);
            g0 = fp[0];
            g1 = fp[1];
            xn = zs[nl.a + kn];
          }
        }
        MT left = shfl_up_v<AR>(carry, width);
        if (li == 0) left = AR::zero();
        MT out = AR::zero();
        if (ok) {
          out = line_row<AR, WT, false>(x, f0, f1, left, carry, WT());
          zs[cl.a + k] = out;
        }
        carry = out;
        cl = nl;
        k = kn;
        ok = okn;
        f0 = g0;
        f1 = g1;
        x = xn;
        pc = pn;
      }
    } else {
      const int lhi = tab[3 * j];
      const int llo = j + 1 < P ? tab[3 * (j + 1)] + 1 : 0;
      LineLevel cl = line_level(L, lhi, mem);
      int k = li - cl.lo;
      bool ok = (unsigned)k < (unsigned)cl.w;
      WT b0 = WT(), b1 = WT(), dg = WT();
      MT x = AR::zero();
      if (ok) {
        const WT *bp = reinterpret_cast<const WT *>(pc) + 3 * (cl.t0 + k);
        b0 = bp[0];
        b1 = bp[1];
        dg = bp[2];
        x = zs[cl.a + k];
      }
      for (int l = lhi; l >= llo; --l) {
        const uint8_t *pn = pc + al16(3 * vs * cl.wsum);
        LineLevel nl{};
        int kn = 0;
        bool okn = false;
        WT c0 = WT(), c1 = WT(), cd = WT();
        MT xn = AR::zero();
        if (l - 1 >= llo) {
          nl = line_level(L, l - 1, mem);
          kn = li - nl.lo;
          okn = (unsigned)kn < (unsigned)nl.w;
          if (okn) {
            const WT *bp = reinterpret_cast<const WT *>(pn) + 3 * (nl.t0 + kn);
            c0 = bp[0];
            c1 = bp[1];
            cd = bp[2];
            xn = zs[nl.a + kn];
          }
        }
        MT right = shfl_down_v<AR>(carry, width);
        if (li == width - 1) right = AR::zero();
        MT out = AR::zero();
        if (ok) {
          // U slots in increasing column: (i, j+1) (this lane's line) is
          // on an earlier line than (i+1, j)
          out = line_row<AR, WT, true>(x, b1, b0, carry, right, dg);
          zs[cl.a + k] = out;
        }
        carry = out;
        cl = nl;
        k = kn;
        ok = okn;
        b0 = c0;
        b1 = c1;
        dg = cd;
        x = xn;
        pc = pn;
      }
    }
    // every lane has consumed its reads of this buffer before it is refilled
    __syncwarp();
    if (lane == 0 && j + 2 < P) {
      fence_proxy_async();
      mbar_expect_tx(&bar[sb], (uint32_t)tab[3 * (j + 2) + 2]);
      bulk_load(buf0 + (sb ? m.buf1 : 0), g + tab[3 * (j + 2) + 1],
                (uint32_t)tab[3 * (j + 2) + 2], &bar[sb]);
    }
  }
  __syncwarp();
  if constexpr (MODE == 3) {
    // y of the group's (at most two) subdomains, read once
    const MT y0 = AR::load_y(def_y, m.sub0);
    const MT y1 = m.nsub > 1 ? AR::load_y(def_y, m.sub0 + 1) : y0;
    for (int i = lane; i < nr; i += 32)
      z[m.r0 + i] = AR::add(zs[i], i < m.nr0 ? y0 : y1);
  } else {
    for (int i = lane; i < nr; i += 32) z[m.r0 + i] = zs[i];
  }
}

// Float-float step-form sweeps (kernels.cuh StepMeta) of the mixed
// solver: per step each lane loads one 16-byte index word and its four
// float-pair values, then z[row] = (z[row] - w0 z[c0] - w1 z[c1] - w2 z[c2])
// (* 1/u_ii) with a compensated (Dot2) accumulation whose only serial
// dependence is one FP32 add per term.  Pieces of kStepsPerPiece steps are
// double-buffered through shared memory by TMA as in the FP64 stream
// kernel; z (8-byte entries) stays in shared memory.
template <int MODE>
__global__ void __launch_bounds__(32)
k_ilu0_apply_dd(const StepMeta *__restrict__ meta,
                const uint8_t *__restrict__ rec, const float2 *__restrict__ r,
                float2 *__restrict__ pv, const float2 *__restrict__ v,
                float2 *__restrict__ z, const KScalars *__restrict__ sc,
                int *__restrict__ err) {
  if (sc && sc->done) return;
  constexpr int SB = kStepBytesDd;
  constexpr int PB = kStepsPerPiece * SB;
  extern __shared__ __align__(128) uint8_t smem[];
  __shared__ __align__(8) uint64_t bar[2];
  const StepMeta m = meta[blockIdx.x];
  const int lane = threadIdx.x;
  const int nr = m.nr, nf = m.n_fwd, S = m.n_fwd + m.n_bwd;
  const int P = (S + kStepsPerPiece - 1) / kStepsPerPiece;
  uint8_t *const buf0 = smem;  // buffer b at buf0 + b*PB
  float2 *zs = reinterpret_cast<float2 *>(smem + 2 * PB);
  const uint8_t *g = rec + m.rec_off;
  auto piece_bytes = [&](int j) {
    const int n = S - j * kStepsPerPiece;
    return (uint32_t)((n < kStepsPerPiece ? n : kStepsPerPiece) * SB);
  };
  if (lane == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    for (int j = 0; j < 2 && j < P; ++j) {
      mbar_expect_tx(&bar[j], piece_bytes(j));
      bulk_load(buf0 + j * PB, g + (size_t)j * PB, piece_bytes(j), &bar[j]);
    }
  }
  for (int i = lane; i < nr; i += 32)
    zs[i] = dd_pre_input(MODE, m.r0 + i, r, pv, v, sc);
  if (lane == 0) zs[nr] = make_float2(0.f, 0.f);
  __syncwarp();
  const uint8_t *zb = reinterpret_cast<const uint8_t *>(zs);
  uint8_t *zw = reinterpret_cast<uint8_t *>(zs);
  auto zat = [&](uint32_t off) { return *reinterpret_cast<const float2 *>(zb + off); };
  // one step; the values arrive as two float4 = {w0, w1}, {w2, 1/u_ii}
  auto step = [&](const uint4 &e, const float4 &wa, const float4 &wb,
                  bool bwd) {
    DdAcc acc = dd_acc(zat(e.x));
    dd_acc_fma(acc, make_float2(-wa.x, -wa.y), zat(e.y));
    dd_acc_fma(acc, make_float2(-wa.z, -wa.w), zat(e.z));
    dd_acc_fma(acc, make_float2(-wb.x, -wb.y), zat(e.w));
    float2 out = dd_value(acc);
    if (bwd) out = dd_mul(out, make_float2(wb.z, wb.w));
    *reinterpret_cast<float2 *>(zw + e.x) = out;
    __syncwarp();
  };
  uint32_t phases = 0u;
  int q = 0;  // global step index
  for (int j = 0; j < P; ++j) {
    const int sb = j & 1;
    if (!mbar_wait_bounded(&bar[sb], err, (phases >> sb) & 1u)) {
      if (j + 1 < P)
        mbar_wait_bounded(&bar[sb ^ 1], nullptr, (phases >> (sb ^ 1)) & 1u);
      return;
    }
    phases ^= 1u << sb;
    const uint8_t *pc = buf0 + sb * PB;
    const int ns = (S - q) < kStepsPerPiece ? (S - q) : kStepsPerPiece;
    auto E = [&](int k) {
      return reinterpret_cast<const uint4 *>(pc + k * SB)[lane];
    };
    auto W = [&](int k, int h) {
      return reinterpret_cast<const float4 *>(pc + k * SB + kStepIdxBytes)[2 * lane + h];
    };
    int k = 0;
    for (; k + 1 < ns; k += 2, q += 2) {
      const uint4 e0 = E(k), e1 = E(k + 1);
      const float4 a0 = W(k, 0), b0 = W(k, 1), a1 = W(k + 1, 0), b1 = W(k + 1, 1);
      step(e0, a0, b0, q >= nf);
      step(e1, a1, b1, q + 1 >= nf);
    }
    if (k < ns) {
      step(E(k), W(k, 0), W(k, 1), q >= nf);
      ++q;
    }
    if (lane == 0 && j + 2 < P) {
      fence_proxy_async();
      mbar_expect_tx(&bar[sb], piece_bytes(j + 2));
      bulk_load(buf0 + sb * PB, g + (size_t)(j + 2) * PB, piece_bytes(j + 2),
                &bar[sb]);
    }
  }
  for (int i = lane; i < nr; i += 32) z[m.r0 + i] = zs[i];
}

// Sweeps with the factor records and the vector in global memory, one CTA
// per subdomain, for subdomains too large for the shared-memory forms (one
// global subdomain on a big system) -- slow, but it needs no staging.
template <class VT, class MT, int MODE>
__global__ void k_ilu0_apply_global(const SubMeta *__restrict__ meta,
                                    const uint8_t *__restrict__ rec,
                                    const VT *__restrict__ r,
                                    VT *__restrict__ pv,
                                    const VT *__restrict__ v,
                                    VT *__restrict__ z,
                                    const KScalars *__restrict__ sc_base,
                                    const int32_t *__restrict__ sub_sys) {
  const KScalars *sc =
      sc_base && sub_sys ? sc_base + sub_sys[blockIdx.x] : sc_base;
  if (sc && sc->done) return;
  const SubMeta m = meta[blockIdx.x];
  const uint8_t *base = rec + m.rec_off;
  const uint16_t *lvl = reinterpret_cast<const uint16_t *>(base);
  const uint16_t *cols = reinterpret_cast<const uint16_t *>(base + m.col_off);
  const MT *vals = reinterpret_cast<const MT *>(base + m.val_off);
  VT *zs = z + m.r0;
  const int K = m.K, KL = m.KL, nr = m.nr;
  for (int i = threadIdx.x; i < nr; i += blockDim.x)
    zs[i] = pre_input<VT>(MODE, m.r0 + i, r, pv, v, sc);
  __syncthreads();
  for (int lv = 0; lv < m.nlev; ++lv) {
    const int a = lvl[lv], b = lvl[lv + 1];
    for (int i = a + threadIdx.x; i < b; i += blockDim.x) {
      VT acc = zs[i];
      for (int k = 0; k < KL; ++k) {
        const int c = cols[(size_t)k * nr + i];
        if (c != kPadCol) acc -= (VT)vals[(size_t)k * nr + i] * zs[c];
      }
      zs[i] = acc;
    }
    __syncthreads();
  }
  for (int lv = m.nlev - 1; lv >= 0; --lv) {
    const int a = lvl[lv], b = lvl[lv + 1];
    for (int i = a + threadIdx.x; i < b; i += blockDim.x) {
      VT acc = zs[i];
      for (int k = KL; k < K; ++k) {
        const int c = cols[(size_t)k * nr + i];
        if (c != kPadCol) acc -= (VT)vals[(size_t)k * nr + i] * zs[c];
      }
      zs[i] = acc * (VT)vals[(size_t)K * nr + i];
    }
    __syncthreads();
  }
}

// Packs the FP64 factor into the FP64 streaming record.
template <class MT>
__global__ void k_pack_stream(int n, const int32_t *__restrict__ src,
                              const int32_t *__restrict__ dst,
                              const double *__restrict__ factor,
                              MT *__restrict__ out) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += gridDim.x * blockDim.x)
    out[dst[e]] = (MT)factor[src[e]];
}

// Packs the FP64 factor into the float-float step stream.
__global__ void k_pack_dd(int n, const int32_t *__restrict__ src,
                          const int32_t *__restrict__ dst,
                          const double *__restrict__ factor,
                          float2 *__restrict__ out) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n;
       e += gridDim.x * blockDim.x)
    out[dst[e]] = dd_from(factor[src[e]]);
}

template <class AR, int MODE, int KLT, int KUT>
void launch_stream(const SolverDev &d, size_t smem, const uint8_t *rec,
                   const typename AR::V *r, typename AR::V *pv,
                   const typename AR::V *v, typename AR::V *z,
                   const KScalars *sc, cudaStream_t st) {
  static size_t attr = 0;
  if (smem > 48 * 1024 && attr < smem) {
    cudaFuncSetAttribute(k_ilu0_apply_stream<AR, MODE, KLT, KUT>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    attr = smem;
  }
  launch_pdl(k_ilu0_apply_stream<AR, MODE, KLT, KUT>, d.n_grp, 32, smem, st,
             d.smeta64, rec, r, pv, v, z, sc, d.sub_sys, d.err, d.csum,
             d.def_y);
}

template <class AR, int MODE, class WT>
void launch_line_w(int n_grp, const LineMeta *meta, size_t smem,
                   const SolverDev &d, const uint8_t *rec,
                   const typename AR::V *r, typename AR::V *pv,
                   const typename AR::V *v, typename AR::V *z,
                   const KScalars *sc, cudaStream_t st) {
  // FP32 weights: the line-major form; 8-byte weights: the level-major one
  constexpr bool kLineMajor = sizeof(WT) == 4;
  auto kern = kLineMajor ? k_ilu0_apply_line<AR, MODE, WT>
                         : k_ilu0_apply_line_lv<AR, MODE, WT>;
  static size_t attr = 0;
  if (smem > 48 * 1024 && attr < smem) {
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    attr = smem;
  }
  launch_pdl(kern, n_grp, 32, smem, st, meta, rec, r, pv, v, z, sc, d.err,
             d.csum, d.def_y);
  count_launches(1);
}

// the line form: FP64 records for FP64, float-pair copies for float-float,
// or the FP32-weight records when the mixed solver uses them (n_lgrp32)
template <class AR, int MODE>
void launch_line(const SolverDev &d, const uint8_t *rec,
                 const typename AR::V *r, typename AR::V *pv,
                 const typename AR::V *v, typename AR::V *z,
                 const KScalars *sc, cudaStream_t st) {
  if constexpr (std::is_same<AR, ArithDD>::value) {
    if (d.n_lgrp32 > 0) {
      launch_line_w<AR, MODE, float>(d.n_lgrp32, d.lmeta32, d.lsmem32, d, d.lrec32,
                                     r, pv, v, z, sc, st);
      return;
    }
  }
  launch_line_w<AR, MODE, typename AR::V>(d.n_lgrp, d.lmeta, d.lsmem, d, rec,
                                          r, pv, v, z, sc, st);
}

template <class VT, class MT, int MODE>
void apply_mode(const SolverDev &d, const VT *r, VT *pv, const VT *v, VT *z,
                const KScalars *sc, cudaStream_t st) {
  if (d.n_lgrp > 0 && !d.sub_sys) {
    launch_line<ArithF64, MODE>(d, d.lrec64, r, pv, v, z, sc, st);
    return;
  }
  const size_t smem = d.smem64;
  // compile-time slot counts for the common stencils: quadrilaterals (2/2,
  // any subdomain whose rows have at most 2 L and 2 U entries) and
  // triangles (3/3); padding slots make smaller rows fit
  if (smem && d.max_kl <= 2 && d.max_ku <= 2)
    launch_stream<ArithF64, MODE, 2, 2>(d, smem, d.srec64, r, pv, v, z, sc, st);
  else if (smem && d.max_kl <= 3 && d.max_ku <= 3)
    launch_stream<ArithF64, MODE, 3, 3>(d, smem, d.srec64, r, pv, v, z, sc, st);
  else if (smem)
    launch_stream<ArithF64, MODE, 0, 0>(d, smem, d.srec64, r, pv, v, z, sc, st);
  else
    k_ilu0_apply_global<VT, MT, MODE><<<d.n_sub, 1024, 0, st>>>(
        d.meta64, d.rec64, r, pv, v, z, sc, d.sub_sys);
  count_launches(1);
}

template <int MODE>
void apply_mode_dd(const SolverDev &d, const float2 *r, float2 *pv,
                   const float2 *v, float2 *z, const KScalars *sc,
                   cudaStream_t st) {
  if (d.dd_stream && (d.n_lgrp32 > 0 || (d.n_lgrp > 0 && d.lrec_dds)) &&
      !d.sub_sys) {
    launch_line<ArithDD, MODE>(d, d.lrec_dds, r, pv, v, z, sc, st);
    return;
  }
  if (d.dd_stream) {  // level blobs, float pairs in the FP64 record layout
    const size_t smem = d.smem64;
    if (d.max_kl <= 2 && d.max_ku <= 2)
      launch_stream<ArithDD, MODE, 2, 2>(d, smem, d.srec_dds, r, pv, v, z, sc, st);
    else if (d.max_kl <= 3 && d.max_ku <= 3)
      launch_stream<ArithDD, MODE, 3, 3>(d, smem, d.srec_dds, r, pv, v, z, sc, st);
    else
      launch_stream<ArithDD, MODE, 0, 0>(d, smem, d.srec_dds, r, pv, v, z, sc, st);
    count_launches(1);
    return;
  }
  static size_t attr = 0;
  if (d.smem_dd > 48 * 1024 && attr < d.smem_dd) {
    cudaFuncSetAttribute(k_ilu0_apply_dd<MODE>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)d.smem_dd);
    attr = d.smem_dd;
  }
  k_ilu0_apply_dd<MODE><<<d.n_sub, 32, d.smem_dd, st>>>(
      d.tmeta_dd, d.srec_dd, r, pv, v, z, sc, d.err);
  count_launches(1);
}

}  // namespace

void launch_ilu0_factor(const SolverDev &d, const double *pvals, int *bad,
                        bool to_dd, cudaStream_t st) {
  k_ilu0_factor<<<d.n_sub, 32, 0, st>>>(d.meta64, d.rec64, d.rec_src, pvals,
                                        bad);
  count_launches(1);
  auto grid = [](int n) { return (n + 255) / 256 < 2432 ? (n + 255) / 256 : 2432; };
  if (to_dd && d.n_lpack32 > 0) {  // FP32-weight line records
    k_pack_stream<float><<<grid(d.n_lpack32), 256, 0, st>>>(
        d.n_lpack32, d.lpack32_src, d.lpack32_dst,
        reinterpret_cast<const double *>(d.rec64),
        reinterpret_cast<float *>(d.lrec32));
    count_launches(1);
  }
  if (d.n_lpack > 0) {  // line-form records
    k_pack_stream<double><<<grid(d.n_lpack), 256, 0, st>>>(
        d.n_lpack, d.lpack_src, d.lpack_dst,
        reinterpret_cast<const double *>(d.rec64),
        reinterpret_cast<double *>(d.lrec64));
    count_launches(1);
    if (to_dd && d.lrec_dds) {
      k_pack_dd<<<grid(d.n_lpack), 256, 0, st>>>(
          d.n_lpack, d.lpack_src, d.lpack_dst,
          reinterpret_cast<const double *>(d.rec64),
          reinterpret_cast<float2 *>(d.lrec_dds));
      count_launches(1);
    }
  }
  if (d.n_pack > 0 && d.smem64) {
    k_pack_stream<double><<<grid(d.n_pack), 256, 0, st>>>(
        d.n_pack, d.pack_src, d.pack_dst64,
        reinterpret_cast<const double *>(d.rec64),
        reinterpret_cast<double *>(d.srec64));
    count_launches(1);
  }
  if (to_dd && d.srec_dds && d.n_pack > 0 && d.smem64) {
    k_pack_dd<<<grid(d.n_pack), 256, 0, st>>>(
        d.n_pack, d.pack_src, d.pack_dst64,
        reinterpret_cast<const double *>(d.rec64),
        reinterpret_cast<float2 *>(d.srec_dds));
    count_launches(1);
  }
  if (to_dd && d.n_pack_dd > 0) {
    k_pack_dd<<<grid(d.n_pack_dd), 256, 0, st>>>(
        d.n_pack_dd, d.pack_src_dd, d.pack_dst_dd,
        reinterpret_cast<const double *>(d.rec64),
        reinterpret_cast<float2 *>(d.srec_dd));
    count_launches(1);
  }
}

bool launch_ilu0_apply_def(const SolverDev &d, const double *in, double *z,
                           const KScalars *sc, cudaStream_t st) {
  const size_t smem = d.smem64;
  double *pv = const_cast<double *>(in);  // mode 3 reads it only
  if (d.def_y && d.n_lgrp > 0 && !d.sub_sys) {
    launch_line<ArithF64, 3>(d, d.lrec64, nullptr, pv, nullptr, z, sc, st);
    return true;
  }
  if (!smem || !d.def_y) return false;
  if (d.max_kl <= 2 && d.max_ku <= 2)
    launch_stream<ArithF64, 3, 2, 2>(d, smem, d.srec64, nullptr, pv, nullptr, z, sc, st);
  else if (d.max_kl <= 3 && d.max_ku <= 3)
    launch_stream<ArithF64, 3, 3, 3>(d, smem, d.srec64, nullptr, pv, nullptr, z, sc, st);
  else
    launch_stream<ArithF64, 3, 0, 0>(d, smem, d.srec64, nullptr, pv, nullptr, z, sc, st);
  count_launches(1);
  return true;
}

bool launch_ilu0_apply_def_dd(const SolverDev &d, const float2 *in, float2 *z,
                              const KScalars *sc, cudaStream_t st) {
  if (!d.dd_stream || !d.def_y) return false;
  const size_t smem = d.smem64;
  float2 *pv = const_cast<float2 *>(in);  // mode 3 reads it only
  if ((d.n_lgrp32 > 0 || (d.n_lgrp > 0 && d.lrec_dds)) && !d.sub_sys) {
    launch_line<ArithDD, 3>(d, d.lrec_dds, nullptr, pv, nullptr, z, sc, st);
    return true;
  }
  if (d.max_kl <= 2 && d.max_ku <= 2)
    launch_stream<ArithDD, 3, 2, 2>(d, smem, d.srec_dds, nullptr, pv, nullptr, z, sc, st);
  else if (d.max_kl <= 3 && d.max_ku <= 3)
    launch_stream<ArithDD, 3, 3, 3>(d, smem, d.srec_dds, nullptr, pv, nullptr, z, sc, st);
  else
    launch_stream<ArithDD, 3, 0, 0>(d, smem, d.srec_dds, nullptr, pv, nullptr, z, sc, st);
  count_launches(1);
  return true;
}

void launch_ilu0_apply_dd(int mode, const SolverDev &d, const float2 *r,
                          float2 *pv, const float2 *v, float2 *z,
                          const KScalars *sc, cudaStream_t st) {
  if (mode == 0) apply_mode_dd<0>(d, r, pv, v, z, sc, st);
  else if (mode == 1) apply_mode_dd<1>(d, r, pv, v, z, sc, st);
  else apply_mode_dd<2>(d, r, pv, v, z, sc, st);
}

template <class VT, class MT>
void launch_ilu0_apply(int mode, const SolverDev &d, const VT *r, VT *pv,
                       const VT *v, VT *z, const KScalars *sc,
                       cudaStream_t st) {
  if (mode == 0) apply_mode<VT, MT, 0>(d, r, pv, v, z, sc, st);
  else if (mode == 1) apply_mode<VT, MT, 1>(d, r, pv, v, z, sc, st);
  else apply_mode<VT, MT, 2>(d, r, pv, v, z, sc, st);
}

template <class VT, class MT>
void launch_precond(int precond, int mode, const SolverDev &d,
                    const MT *jdinv, const VT *r, VT *pv, const VT *v, VT *z,
                    const KScalars *sc, cudaStream_t st) {
  if (precond == PG_PREC_ILU0)
    launch_ilu0_apply<VT, MT>(mode, d, r, pv, v, z, sc, st);
  else
    launch_diag_apply<VT, MT>(mode, d, precond == PG_PREC_JACOBI ? jdinv : nullptr,
                              r, pv, v, z, sc, st);
}

template void launch_precond<double, double>(int, int, const SolverDev &,
                                             const double *, const double *,
                                             double *, const double *,
                                             double *, const KScalars *,
                                             cudaStream_t);
}  // namespace pg
