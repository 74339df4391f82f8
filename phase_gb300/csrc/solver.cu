// The SparseMatrixSolver replacement: sparsity analysis caching, value
// permutation, ILU(0) factorisation and the device-resident BiCGStab loop
// with reliable residual updates: in FP64 (PG_FP64), or with the whole
// iteration in float-float arithmetic on the FP32 pipes and the FP64 true
// residual at every reliable update (PG_MIXED).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "internal.h"
#include "kernels.cuh"
#include "lu.h"

using namespace pg;

namespace {

__global__ void k_count_diff(int64_t n, const int32_t *__restrict__ a,
                             const int32_t *__restrict__ b,
                             unsigned int *__restrict__ diff) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    if (a[i] != b[i]) {
      atomicAdd(diff, 1u);
      return;
    }
}

// deterministic non-zero contents for kernel timing
__global__ void k_fill_profile(int64_t n, double *__restrict__ a,
                               float *__restrict__ b, int salt) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double v = 1.0 + 0.25 * sinf(0.001f * (float)(i % 100003) + salt);
    if (a) a[i] = v;
    if (b) b[i] = (float)v;
  }
}

}  // namespace

constexpr size_t kMaxApplySmem = 200 * 1024;

struct pg_solver {
  pg_solver_cfg cfg{};
  int64_t rank = 0;
  // analysis
  Analysis a;
  bool analysed = false;
  uint64_t eqn_pattern = 0;  // pattern id of a device equation, 0 = host CSR
  DevBuf<int32_t> perm, prp, pci, psrc, dup_dst, dup_src, rec_src;
  // sliced ELLPACK copy of the matrix for the FP64 SpMVs (PG_FP64 solvers)
  DevBuf<int32_t> sell_ptr, sell_col, sell_src;
  DevBuf<double> sell_val;
  bool sell_on = false;
  int sell_w = 0;  // widest slice
  DevBuf<SubMeta> meta64;
  DevBuf<uint8_t> rec64;
  DevBuf<StreamMeta> smeta64;
  DevBuf<StepMeta> tmeta_dd;
  DevBuf<uint8_t> srec64, srec_dd, srec_dds;
  int dd_stream = -1;  // mixed ILU sweep: -1 not chosen, 0 steps, 1 stream
  DevBuf<int32_t> pack_src, pack_dst64, pack_src_dd, pack_dst_dd;
  // line form of the sweep records (structured blocks)
  DevBuf<LineMeta> lmeta;
  DevBuf<uint8_t> lrec64, lrec_dds;
  DevBuf<int32_t> lpack_src, lpack_dst;
  DevBuf<LineMeta> lmeta32;  // FP32 weights (mixed_sweep 3)
  DevBuf<uint8_t> lrec32;
  DevBuf<int32_t> lpack32_src, lpack32_dst;
  bool line_sweep = true;  // PG_LINE_SWEEP=0 at the analysis: stream kernel
  // the device equation of the last hand-over and its assembly count
  const pg_eqn *eqn_src = nullptr;
  uint64_t eqn_version = 0;
  // the factorisation (and coarse inverse) matches the current values: a
  // solve after a right-hand-side-only hand-over does not redo it
  bool factored = false;
  // TFQMR / GMRES work vectors (allocated on first use): three more
  // vectors, the GMRES basis ((restart + 1) x n), dot-product scratch
  DevBuf<double> k1, k2, k3, kV, kpart, kdot;
  DevBuf<int> err;
  DevBuf<int32_t> raw_rp, raw_ci, st_rp, st_ci;
  std::vector<double> row_x, row_y;  // pg_solver_set_row_coords hint
  DevBuf<double> st_vals, st_vec;
  DevBuf<unsigned int> diff;
  // values and factors
  DevBuf<double> pvals, jdinv;
  // Krylov vectors (permuted order)
  DevBuf<double> b, x, r, rh, p, v, ph, s, sh, t, xout;
  // float-float matrix, Jacobi diagonal and Krylov vectors of PG_MIXED
  DevBuf<float2> pvals_dd, jdinv_dd;
  DevBuf<float2> xd, rd, rhd, pd, vd, phd, sd, shd, td;
  // reductions and scalars
  DevBuf<double> partials;
  DevBuf<unsigned int> ticket;
  DevBuf<KScalars> sc;
  DevBuf<int> bad;
  KScalars *sc_host = nullptr;
  int *bad_host = nullptr;
  unsigned int *diff_host = nullptr;
  bool have_rhs = false, have_x = false, have_vals = false;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  int red_grid = 1;
  // CUDA graphs of one chunk of BiCGStab iterations (FP64, float-float);
  // kernel
  // arguments are fixed device pointers, so a graph stays valid until the
  // buffers are reallocated by a new analysis
  // [0] FP64, [1] float-float; [2], [3] the same without the coarse
  // correction (the warm-up iterations while the coarse inverse is built);
  // [4], [5] as [0], [1] with the second coarse-inverse buffer
  cudaGraphExec_t chunk_graph[6] = {};
  int chunk_launches[6] = {};  // kernels in one replay of each graph
  // pg_solver_trace_kernels: an event after every launch group of the
  // Krylov loop (chunks launched directly, not replayed), each interval
  // booked to the kind of the group that ends it
  struct KernelTrace {
    bool on = false;
    std::vector<cudaEvent_t> ev;
    std::vector<int8_t> kind;
    size_t used = 0;
    int64_t dropped = 0;
  } kt;
  // two-level Schwarz coarse space (cfg.coarse): structure, the dense
  // coarse matrix / its inverse, elimination buffers, subdomain sums and the
  // graph of the K elimination steps
  bool coarse_on = false;
  bool coarse_use = true;   // the Krylov drivers apply the coarse correction
  bool batch_mode = false;  // inner solver of a pg_batch (its own coarse space)
  // the coarse matrix and its inverse are built on side2 beside the first
  // (one-level) iterations; ev_coarse marks them done
  cudaStream_t side2 = nullptr;
  cudaEvent_t ev_cvals = nullptr, ev_coarse = nullptr;
  bool coarse_pending = false;
  DevBuf<int32_t> c_sub_ptr, c_cptr, c_cnb;
  DevBuf<uint8_t> c_slot;
  DevBuf<float> c_ac, c_dg0, c_pinv, c_W, c_V, c_C;
  DevBuf<float2> c_sum;
  DevBuf<int32_t> c_azp, c_azj;
  DevBuf<uint8_t> c_azslot;
  DevBuf<double> c_azv, c_y, c_tmp;
  DevBuf<float2> c_azv_dd, c_y_dd, c_tmp_dd;
  cudaGraphExec_t gj_graph = nullptr;
  // the coarse inverse through the sparse LU of A_c (nested dissection,
  // FP64 factorisation, FP32 dense inverse): built at the analysis when
  // every front of A_c's pattern is small; otherwise (or with
  // PG_COARSE_GJ=1) the blocked Gauss-Jordan inversion runs
  pg_lu *c_lu = nullptr;
  DevBuf<double> c_vals;
  // cfg.coarse_warm = -2: a solve applies the previous factorisation's
  // inverse while the new one is built on side2 into the other buffer
  // (c_ac / c_ac2, one Gauss-Jordan graph each); a join makes the new one
  // current
  DevBuf<float> c_ac2;
  cudaGraphExec_t gj_graph2 = nullptr;
  int ac_ready = 0;      // the buffer the Krylov drivers apply
  int ac_next = -1;      // the buffer being inverted on side2 (-1: none)
  bool ac_valid = false; // ac_ready holds an inverse for this analysis
  float *ac_buf(int b) const { return b ? c_ac2.p : c_ac.p; }
  cudaGraphExec_t *gj_graph_of(int b) { return b ? &gj_graph2 : &gj_graph; }

  void drop_graphs() {
    for (auto &g : chunk_graph)
      if (g) {
        cudaGraphExecDestroy(g);
        g = nullptr;
      }
    for (cudaGraphExec_t *g : {&gj_graph, &gj_graph2})
      if (*g) {
        cudaGraphExecDestroy(*g);
        *g = nullptr;
      }
  }

  CoarseDev coarse() const {
    CoarseDev c;
    if (!coarse_on || !coarse_use) return c;
    c.K = a.n_sub;
    c.max_cnb = a.max_cnb;
    c.sub_ptr = c_sub_ptr.p;
    c.cptr = c_cptr.p;
    c.cnb = c_cnb.p;
    c.cslot = c_slot.p;
    c.ac = ac_buf(ac_ready);
    c.dg0 = c_dg0.p;
    c.pinv = c_pinv.p;
    c.W = c_W.p;
    c.V = c_V.p;
    c.C = c_C.p;
    c.csum = c_sum.p;
    c.azp = c_azp.p;
    c.azj = c_azj.p;
    c.azslot = c_azslot.p;
    c.azv = c_azv.p;
    c.y = c_y.p;
    c.tmp = c_tmp.p;
    c.azv_dd = c_azv_dd.p;
    c.y_dd = c_y_dd.p;
    c.tmp_dd = c_tmp_dd.p;
    return c;
  }

  // the factorisation of the last hand-over runs on `side` (started by
  // set_eqn/set_csr) while the caller prepares the guess; solve waits on
  // ev_fact
  cudaStream_t side = nullptr;
  cudaEvent_t ev_vals = nullptr, ev_fact = nullptr;
  bool fact_pending = false;

  ~pg_solver() {
    if (side) {
      cudaStreamSynchronize(side);
      cudaStreamDestroy(side);
    }
    if (side2) {
      cudaStreamSynchronize(side2);
      cudaStreamDestroy(side2);
    }
    if (ev_vals) cudaEventDestroy(ev_vals);
    if (ev_fact) cudaEventDestroy(ev_fact);
    if (ev_cvals) cudaEventDestroy(ev_cvals);
    if (ev_coarse) cudaEventDestroy(ev_coarse);
    drop_graphs();
    if (c_lu) pg_lu_destroy(c_lu);
    if (sc_host) cudaFreeHost(sc_host);
    if (bad_host) cudaFreeHost(bad_host);
    if (diff_host) cudaFreeHost(diff_host);
    for (auto &e : ev)
      if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : kt.ev) cudaEventDestroy(e);
  }

  SolverDev dev() const {
    SolverDev d;
    d.n = (int)a.n;
    d.nnz = (int)a.nnz;
    d.n_sub = a.n_sub;
    d.prp = prp.p;
    d.pci = pci.p;
    if (sell_on) {
      d.sell_ptr = sell_ptr.p;
      d.sell_col = sell_col.p;
      d.sell_val = sell_val.p;
      d.sell_w = sell_w;
    }
    d.meta64 = meta64.p;
    d.rec64 = rec64.p;
    d.rec_src = rec_src.p;
    // the streamed (TMA) apply needs header + 2 pieces + the subdomain's
    // vector in shared memory; otherwise the global-memory sweep is used
    d.smem64 = a.ssmem64 <= kMaxApplySmem ? a.ssmem64 : 0;
    d.smeta64 = smeta64.p;
    d.n_grp = a.n_grp;
    d.srec64 = srec64.p;
    d.pack_src = pack_src.p;
    d.pack_dst64 = pack_dst64.p;
    d.n_pack = (int)a.pack_src.size();
    d.use_steps = a.use_steps ? 1 : 0;
    d.smem_dd = a.use_steps && a.ssmem_dd <= kMaxApplySmem ? a.ssmem_dd : 0;
    d.tmeta_dd = tmeta_dd.p;
    d.srec_dd = srec_dd.p;
    d.pack_src_dd = pack_src_dd.p;
    d.pack_dst_dd = pack_dst_dd.p;
    d.n_pack_dd = (int)a.pack_src_dd.size();
    d.srec_dds = srec_dds.p;
    d.dd_stream = dd_stream == 1 ? 1 : 0;
    d.max_kl = a.max_kl;
    d.max_ku = a.max_ku;
    d.err = err.p;
    d.sub_sys = nullptr;
    d.csum = coarse_on ? c_sum.p : nullptr;
    d.def_y = nullptr;
    const bool line =
        line_sweep && !a.lmeta.empty() && a.lsmem <= kMaxApplySmem;
    d.n_lgrp = line ? (int)a.lmeta.size() : 0;
    d.lmeta = lmeta.p;
    d.lrec64 = lrec64.p;
    d.lrec_dds = cfg.precision == PG_MIXED ? lrec_dds.p : nullptr;
    d.lsmem = a.lsmem;
    d.lpack_src = lpack_src.p;
    d.lpack_dst = lpack_dst.p;
    d.n_lpack = line ? (int)a.lpack_src.size() : 0;
    const bool line32 = line && cfg.precision == PG_MIXED &&
                        cfg.mixed_sweep == 3 && !a.lmeta32.empty() &&
                        a.lsmem32 <= kMaxApplySmem;
    d.n_lgrp32 = line32 ? (int)a.lmeta32.size() : 0;
    d.lmeta32 = lmeta32.p;
    d.lrec32 = lrec32.p;
    d.lsmem32 = a.lsmem32;
    d.lpack32_src = lpack32_src.p;
    d.lpack32_dst = lpack32_dst.p;
    d.n_lpack32 = line32 ? (int)a.lpack32_src.size() : 0;
    return d;
  }
  RedWork red() const { return RedWork{partials.p, ticket.p, red_grid, err.p}; }
};

namespace {

// CTAs of the reducing vector kernels (grid-stride loops): every thread
// ends with a warp/block reduction whose FP64 shuffles and adds are not
// free on GB300's FP64 pipe, so fewer threads with more rows each win until
// memory parallelism runs short.  PG_RED_GRID overrides the cap.
int red_grid_cap() {
  static const int cap = [] {
    const char *e = std::getenv("PG_RED_GRID");
    const int v = e ? std::atoi(e) : 0;
    return v > 0 ? v : 1216;
  }();
  return cap;
}

constexpr int kMaxCoarseK = 2048;  // the coarse matrix is K x K, dense
// by default, coarse spaces of at least kCoarseStagedK subdomains that are
// inverted by Gauss-Jordan elimination (~1.5 ms at 2048) are inverted
// beside kCoarseWarmIters one-level iterations; an inverse built through
// the sparse LU (well under a millisecond) is waited for (cfg.coarse_warm
// overrides both)
constexpr int kCoarseStagedK = 1024;
constexpr int kCoarseWarmIters = 16;

// Schwarz subdomain size for the analysis: the configured one, else 1024
// rows for the one-level preconditioner and 512 with a coarse space (the
// coarse correction carries the global coupling, so smaller, faster ILU(0)
// blocks pay), enlarged so the coarse matrix stays within kMaxCoarseK;
// -1 (one subdomain) for the other preconditioners
int subdomain_rows_for(const pg_solver_cfg &c, int64_t n) {
  if (c.precond != PG_PREC_ILU0) return -1;
  if (c.subdomain_rows) return c.subdomain_rows;
  if (!c.coarse) return 1024;
  return (int)std::max<int64_t>(512, (n + kMaxCoarseK - 1) / kMaxCoarseK);
}

// level of fill of the ILU blocks (ILU preconditioner only)
int ilu_fill_of(const pg_solver_cfg &c) {
  return c.precond == PG_PREC_ILU0 ? c.ilu_fill : 0;
}

int upload_analysis(pg_solver *s) {
  if (s->fact_pending || s->coarse_pending) {  // buffers are about to move
    PG_CUDA(cudaStreamSynchronize(s->side));
    PG_CUDA(cudaStreamSynchronize(s->side2));
    s->fact_pending = false;
    s->coarse_pending = false;
  }
  const Analysis &a = s->a;
  cudaError_t e = cudaSuccess;
  auto up = [&](auto &buf, const auto &vec) {
    if (e == cudaSuccess) e = buf.upload(vec);
  };
  up(s->perm, a.perm);
  up(s->prp, a.prp);
  up(s->pci, a.pci);
  s->sell_on = s->cfg.precision == PG_FP64 && !s->batch_mode &&
               !a.sell_ptr.empty();
  if (s->sell_on) {
    up(s->sell_ptr, a.sell_ptr);
    up(s->sell_col, a.sell_col);
    up(s->sell_src, a.sell_src);
    if (e == cudaSuccess) e = s->sell_val.reserve(a.sell_col.size());
    s->sell_w = 0;
    for (size_t sl = 0; sl + 1 < a.sell_ptr.size(); ++sl)
      s->sell_w = std::max<int>(s->sell_w, (a.sell_ptr[sl + 1] - a.sell_ptr[sl]) / 32);
  }
  up(s->psrc, a.psrc);
  up(s->dup_dst, a.dup_dst);
  up(s->dup_src, a.dup_src);
  up(s->rec_src, a.rec_src);
  up(s->meta64, a.meta64);
  up(s->rec64, a.rec64);
  up(s->smeta64, a.smeta64);
  up(s->srec64, a.srec64);
  up(s->pack_src, a.pack_src);
  up(s->pack_dst64, a.pack_dst64);
  up(s->tmeta_dd, a.tmeta_dd);
  up(s->srec_dd, a.srec_dd);
  s->dd_stream = -1;
  if (s->cfg.precision == PG_MIXED) up(s->srec_dds, a.srec64);  // static parts
  up(s->pack_src_dd, a.pack_src_dd);
  up(s->pack_dst_dd, a.pack_dst_dd);
  {
    const char *e = std::getenv("PG_LINE_SWEEP");
    s->line_sweep = !(e && e[0] == '0');
  }
  up(s->lmeta, a.lmeta);
  up(s->lrec64, a.lrec);
  if (s->cfg.precision == PG_MIXED) up(s->lrec_dds, a.lrec);  // static parts
  up(s->lpack_src, a.lpack_src);
  up(s->lpack_dst, a.lpack_dst);
  if (s->cfg.precision == PG_MIXED && s->cfg.mixed_sweep == 3) {
    up(s->lmeta32, a.lmeta32);
    up(s->lrec32, a.lrec32);
    up(s->lpack32_src, a.lpack32_src);
    up(s->lpack32_dst, a.lpack32_dst);
  }

  if (e == cudaSuccess) e = s->err.zero(1);
  const size_t n = a.n, nnz = a.nnz;
  for (DevBuf<double> *bf : {&s->b, &s->x, &s->r, &s->rh, &s->p, &s->v,
                             &s->ph, &s->s, &s->sh, &s->t, &s->xout,
                             &s->jdinv})
    if (e == cudaSuccess) e = bf->reserve(n);
  if (e == cudaSuccess) e = s->pvals.reserve(nnz);
  if (s->cfg.precision == PG_MIXED) {
    for (DevBuf<float2> *bf : {&s->xd, &s->rd, &s->rhd, &s->pd, &s->vd,
                               &s->phd, &s->sd, &s->shd, &s->td, &s->jdinv_dd})
      if (e == cudaSuccess) e = bf->reserve(n);
    if (e == cudaSuccess) e = s->pvals_dd.reserve(nnz);
  }
  s->drop_graphs();
  s->coarse_on = false;
  if (s->cfg.coarse && !s->batch_mode && s->cfg.precond == PG_PREC_ILU0 &&
      a.n_sub > 1) {
    PG_CHECK_ARG(a.n_sub <= kMaxCoarseK,
                 "coarse correction: more than 2048 subdomains (raise "
                 "subdomain_rows)");
    PG_CHECK_ARG(a.max_cnb <= kMaxCoarseNb,
                 "coarse correction: a subdomain couples to more than 32 "
                 "others");
    const size_t K = a.n_sub;
    up(s->c_sub_ptr, a.sub_ptr);
    up(s->c_cptr, a.cptr);
    up(s->c_cnb, a.cnb);
    up(s->c_slot, a.cslot);
    if (e == cudaSuccess) e = s->c_ac.reserve(K * K);
    if (e == cudaSuccess && s->cfg.coarse_warm == -2) e = s->c_ac2.reserve(K * K);
    s->ac_ready = 0;
    s->ac_next = -1;
    s->ac_valid = false;
    if (e == cudaSuccess) e = s->c_dg0.reserve(K);
    if (e == cudaSuccess) e = s->c_pinv.reserve(2 * 32 * 32);  // two steps
    for (DevBuf<float> *bf : {&s->c_W, &s->c_V, &s->c_C})
      if (e == cudaSuccess) e = bf->reserve(32 * K);
    if (e == cudaSuccess) e = s->c_sum.reserve(K);
    if (s->c_lu) {
      pg_lu_destroy(s->c_lu);
      s->c_lu = nullptr;
    }
    const char *gj = std::getenv("PG_COARSE_GJ");
    if (e == cudaSuccess && !(gj && gj[0] == '1')) {
      int rc = lu_inverse_setup((int64_t)K, a.cptr.data(), a.cnb.data(), &s->c_lu);
      if (rc) return rc;
      if (s->c_lu) e = s->c_vals.reserve(a.cnb.size());
    }
    if (s->cfg.coarse == 2) {
      up(s->c_azp, a.azp);
      up(s->c_azj, a.azj);
      up(s->c_azslot, a.azslot);
      if (e == cudaSuccess) e = s->c_azv.reserve(a.azj.size());
      if (e == cudaSuccess) e = s->c_y.reserve(K);
      if (e == cudaSuccess) e = s->c_tmp.reserve(a.n);
      if (s->cfg.precision == PG_MIXED) {
        if (e == cudaSuccess) e = s->c_azv_dd.reserve(a.azj.size());
        if (e == cudaSuccess) e = s->c_y_dd.reserve(K);
        if (e == cudaSuccess) e = s->c_tmp_dd.reserve(a.n);
      }
    }
    s->coarse_on = true;
  }
  s->red_grid = (int)std::min<int64_t>(red_grid_cap(), (n + kVecBlock - 1) / kVecBlock);
  if (s->red_grid < 1) s->red_grid = 1;
  if (e == cudaSuccess) e = s->partials.reserve((size_t)kMaxDots * s->red_grid);
  if (e == cudaSuccess) e = s->ticket.zero(1);
  if (e == cudaSuccess) e = s->sc.reserve(1);
  if (e == cudaSuccess) e = s->bad.reserve(1);
  if (e == cudaSuccess) e = s->diff.reserve(1);
  if (e != cudaSuccess) return cuda_fail(e, "solver analysis upload", __FILE__, __LINE__);
  s->analysed = true;
  s->have_x = false;
  s->have_rhs = false;
  s->factored = false;
  return PG_OK;
}

int ensure_host_state(pg_solver *s) {
  if (!s->sc_host) PG_CUDA(cudaMallocHost((void **)&s->sc_host, sizeof(KScalars)));
  if (!s->bad_host) PG_CUDA(cudaMallocHost((void **)&s->bad_host, sizeof(int)));
  if (!s->diff_host) PG_CUDA(cudaMallocHost((void **)&s->diff_host, sizeof(unsigned)));
  for (auto &e : s->ev)
    if (!e) PG_CUDA(cudaEventCreate(&e));
  // the factorisation streams run at the highest priority: their kernels
  // form short dependent chains (the coarse inverse is ~130 launches) that
  // must not queue behind the blocks of whatever the library stream runs
  // meanwhile (a network's inference, one-level iterations)
  int prio_lo = 0, prio_hi = 0;
  PG_CUDA(cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi));
  if (!s->side)
    PG_CUDA(cudaStreamCreateWithPriority(&s->side, cudaStreamNonBlocking, prio_hi));
  if (!s->ev_vals) PG_CUDA(cudaEventCreateWithFlags(&s->ev_vals, cudaEventDisableTiming));
  if (!s->ev_fact) PG_CUDA(cudaEventCreateWithFlags(&s->ev_fact, cudaEventDisableTiming));
  if (!s->side2)
    PG_CUDA(cudaStreamCreateWithPriority(&s->side2, cudaStreamNonBlocking, prio_hi));
  if (!s->ev_cvals) PG_CUDA(cudaEventCreateWithFlags(&s->ev_cvals, cudaEventDisableTiming));
  if (!s->ev_coarse) PG_CUDA(cudaEventCreateWithFlags(&s->ev_coarse, cudaEventDisableTiming));
  return PG_OK;
}

// The library stream waits for the coarse matrix and inverse built on side2.
int join_coarse(pg_solver *s) {
  if (!s->coarse_pending) return PG_OK;
  PG_CUDA(cudaStreamWaitEvent(stream(), s->ev_coarse, 0));
  s->coarse_pending = false;
  if (s->ac_next >= 0) s->ac_ready = s->ac_next;  // the new inverse is current
  s->ac_next = -1;
  s->ac_valid = true;
  return PG_OK;
}

// The library stream waits for a factorisation still running on the side
// stream (before anything on it reads or rewrites the values or factors).
int join_factor(pg_solver *s) {
  if (!s->fact_pending) return PG_OK;
  PG_CUDA(cudaStreamWaitEvent(stream(), s->ev_fact, 0));
  s->fact_pending = false;
  return PG_OK;
}

// one chunk = kChunk BiCGStab iterations (5 kernels each, 7 with the coarse
// correction); captured once into
// a CUDA graph after the first direct chunk and replayed
constexpr int kChunk = 8;
constexpr double kDelta2 = 1e-4;  // reliable update when rr < kDelta2 * rr_ref
constexpr int kMaxRestarts = 50;
// float-float solver: hand over to FP64 when the true residual norm has not
// fallen 10x in kDdStallIters iterations or after kDdMaxRestarts breakdowns
constexpr int kDdStallIters = 1200;
constexpr int kDdMaxRestarts = 4;
constexpr int kDdStalled = -1000;  // internal status of run_bicgstab_dd

// PG_SOLVER_TRACE=1 prints the Krylov scalars at every chunk boundary
bool trace_enabled() {
  static const int on = [] {
    const char *e = std::getenv("PG_SOLVER_TRACE");
    return e && e[0] == '1' ? 1 : 0;
  }();
  return on != 0;
}

// Kernel trace (pg_solver_trace_kernels): records an event on st that
// ends an interval of the given kind (PG_KT_*; -1 opens a new run of
// intervals after a host wait).  Events come from a pool that grows by 256
// up to kKtMaxEvents; past that the rest of the solve is not timed.
constexpr size_t kKtMaxEvents = 1 << 16;
void kt_mark(pg_solver *s, int kind, cudaStream_t st) {
  auto &t = s->kt;
  if (!t.on) return;
  if (t.dropped) {
    ++t.dropped;
    return;
  }
  if (t.used == t.ev.size()) {
    for (int i = 0; i < 256 && t.ev.size() < kKtMaxEvents; ++i) {
      cudaEvent_t e;
      if (cudaEventCreate(&e) != cudaSuccess) break;
      t.ev.push_back(e);
      t.kind.push_back(-1);
    }
    if (t.used == t.ev.size()) {
      ++t.dropped;
      return;
    }
  }
  if (cudaEventRecord(t.ev[t.used], st) != cudaSuccess) {
    ++t.dropped;
    return;
  }
  t.kind[t.used++] = (int8_t)kind;
}

// Replays the captured chunk graph (capturing it on the second call); with
// the kernel trace on, every chunk is launched directly.
template <class F>
int run_chunk(cudaGraphExec_t &gexec, int &n_launch, bool &direct_done,
              F &&chunk, bool direct = false) {
  cudaStream_t st = stream();
  if (direct) {
    chunk();
  } else if (gexec) {
    PG_CUDA(cudaGraphLaunch(gexec, st));
    count_launches(n_launch);
  } else if (direct_done) {
    cudaGraph_t graph = nullptr;
    PG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
    const uint64_t before = launch_count();
    chunk();  // launches are counted here, executed once below
    n_launch = (int)(launch_count() - before);
    PG_CUDA(cudaStreamEndCapture(st, &graph));
    cudaError_t ge = cudaGraphInstantiate(&gexec, graph, 0);
    cudaGraphDestroy(graph);
    PG_CUDA(ge);
    PG_CUDA(cudaGraphLaunch(gexec, st));
  } else {
    chunk();
    direct_done = true;
  }
  PG_CUDA(cudaGetLastError());
  return PG_OK;
}

inline int grid_for(int64_t n) {
  return (int)std::min<int64_t>(1216, std::max<int64_t>(1, (n + 255) / 256));
}

// Right-preconditioned BiCGStab on the permuted system (b, x), as Belos
// BICGSTAB with an Ifpack2 RILUK right preconditioner
// (TrilinosBelosSparseMatrixSolver.cpp:18-29,44-86), with reliable residual
// updates (van der Vorst & Ye 2000): at a chunk boundary where the recursive
// residual has dropped by kDelta2 since the last update, or has met the
// tolerance, the FP64 true residual b - A x replaces it; the search
// directions are kept unless the recurrence broke down, in which case the
// iteration restarts from x with a fresh shadow residual.  Convergence is
// only ever declared on the true residual.
int run_bicgstab(pg_solver *s, double tol, int max_iters, int *iters,
                 int *updates, double *bb_out) {
  cudaStream_t st = stream();
  const SolverDev d = s->dev();
  const RedWork w = s->red();
  double *const val = s->pvals.p, *const jd = s->jdinv.p;
  double *const x = s->x.p, *const r = s->r.p, *const rh = s->rh.p;
  double *const p = s->p.p, *const v = s->v.p, *const ph = s->ph.p;
  double *const ss = s->s.p, *const sh = s->sh.p, *const t = s->t.p;
  const CoarseDev cdev = s->coarse();
  const bool ilu_stream = s->cfg.precond == PG_PREC_ILU0 && d.smem64 > 0;
  SolverDev d0 = d;  // the deflated form's sweep needs no subdomain sums
  d0.csum = nullptr;
  SolverDev d3 = d0;  // ... and adds y on output (mode 3)
  d3.def_y = cdev.y;
  auto precond = [&](int mode, double *pv, double *z) {
    if (cdev.K && s->cfg.coarse == 2) {
      // A-DEF1: y = A_c^-1 Z^T p, z = B (p - A Z y) + Z y; the streamed
      // sweep adds y as it writes z
      launch_def_pre(cdev, mode, r, pv, v, s->sc.p, st);
      launch_def_in(cdev, d.n, pv, cdev.tmp, s->sc.p, st);
      kt_mark(s, PG_KT_COARSE, st);
      if (s->cfg.precond == PG_PREC_ILU0 &&
          launch_ilu0_apply_def(d3, cdev.tmp, z, s->sc.p, st)) {
        kt_mark(s, PG_KT_SWEEP, st);
        return;
      }
      launch_precond<double, double>(s->cfg.precond, 0, d0, jd, r, cdev.tmp,
                                     v, z, s->sc.p, st);
      kt_mark(s, PG_KT_SWEEP, st);
      launch_coarse_add(cdev, z, s->sc.p, st);
      kt_mark(s, PG_KT_COARSE, st);
      return;
    }
    launch_precond<double, double>(s->cfg.precond, mode, d, jd, r, pv, v, z,
                                   s->sc.p, st);
    kt_mark(s, PG_KT_SWEEP, st);
    // the input (p or s) is in pv after the fused update; the streamed
    // ILU(0) sweep has summed it per subdomain already
    if (cdev.K) {
      launch_coarse_apply(cdev, pv, z, ilu_stream, s->sc.p, st);
      kt_mark(s, PG_KT_COARSE, st);
    }
  };
  auto chunk = [&]() {
    kt_mark(s, -1, st);
    for (int c = 0; c < kChunk; ++c) {
      precond(1, p, ph);
      launch_spmv_v<double, double>(d, val, ph, v, rh, s->sc.p, w, st);
      kt_mark(s, PG_KT_SPMV, st);
      precond(2, ss, sh);
      launch_spmv_t<double, double>(d, val, sh, t, ss, s->sc.p, w, st);
      kt_mark(s, PG_KT_SPMV, st);
      launch_update<double>(d.n, x, r, ph, sh, ss, t, rh, s->sc.p, w, st);
      kt_mark(s, PG_KT_UPDATE, st);
    }
  };
  auto read_scalars = [&]() -> int {
    PG_CUDA(cudaMemcpyAsync(s->sc_host, s->sc.p, sizeof(KScalars),
                            cudaMemcpyDeviceToHost, st));
    PG_CUDA(cudaStreamSynchronize(st));
    return PG_OK;
  };
  KScalars init{};
  init.tol2 = tol * tol;
  init.max_iter = max_iters;
  *s->sc_host = init;
  PG_CUDA(cudaMemcpyAsync(s->sc.p, s->sc_host, sizeof(KScalars),
                          cudaMemcpyHostToDevice, st));
  // ||b||^2 and r = b - A x, then a fresh start
  launch_true_residual(d, val, s->b.p, nullptr, nullptr, s->sc.p, w, st);
  int rc = read_scalars();
  if (rc) return rc;
  const double bb = s->sc_host->rr_true;
  *bb_out = bb;  // unscaled ||b||^2 for the caller's final check
  *iters = 0;
  *updates = 0;
  if (!std::isfinite(bb)) return PG_NON_FINITE;
  if (bb == 0.) {
    PG_CUDA(cudaMemsetAsync(x, 0, d.n * sizeof(double), st));
    return PG_OK;
  }
  init.bb = bb;
  init.rr_true = bb;
  *s->sc_host = init;
  PG_CUDA(cudaMemcpyAsync(s->sc.p, s->sc_host, sizeof(KScalars),
                          cudaMemcpyHostToDevice, st));
  launch_true_residual(d, val, s->b.p, x, r, s->sc.p, w, st);
  launch_init_from_r(d.n, r, rh, p, v, s->sc.p, w, st);
  if ((rc = read_scalars())) return rc;
  if (s->sc_host->status == PG_NON_FINITE) return PG_NON_FINITE;
  if (s->sc_host->rr_true <= init.tol2 * bb) return PG_OK;
  double rr_ref = s->sc_host->rr_true;
  int restarts = 0;
  const int slot = cdev.K ? (s->ac_ready ? 4 : 0) : 2;
  cudaGraphExec_t &gexec = s->chunk_graph[slot];
  bool direct_done = false;
  for (;;) {
    if ((rc = run_chunk(gexec, s->chunk_launches[slot], direct_done, chunk,
                        s->kt.on)))
      return rc;
    if ((rc = read_scalars())) return rc;
    const KScalars k = *s->sc_host;
    *iters = k.iter;
    if (trace_enabled())
      std::fprintf(stderr,
                   "pg_solver: it %d rr/bb %.3e rho %.3e alpha %.3e omega "
                   "%.3e status %d done %d\n",
                   k.iter, k.rr / bb, k.rho, k.alpha, k.omega, k.status,
                   k.done);
    if (k.status == PG_NON_FINITE) return PG_NON_FINITE;
    if (!k.done && !(k.rr < kDelta2 * rr_ref)) continue;
    // reliable update: r = b - A x in FP64
    launch_true_residual(d, val, s->b.p, x, r, s->sc.p, w, st);
    if ((rc = read_scalars())) return rc;
    const double rr_true = s->sc_host->rr_true;
    ++*updates;
    if (trace_enabled())
      std::fprintf(stderr, "pg_solver: it %d true rr/bb %.3e (%s)\n", k.iter,
                   rr_true / bb, k.status == PG_BREAKDOWN ? "restart" : "replace");
    if (!std::isfinite(rr_true)) return PG_NON_FINITE;
    if (rr_true <= init.tol2 * bb) return PG_OK;
    if (k.iter >= max_iters) return PG_MAX_ITERS;
    if (k.status == PG_BREAKDOWN) {
      if (++restarts > kMaxRestarts) return PG_BREAKDOWN;
      launch_init_from_r(d.n, r, rh, p, v, s->sc.p, w, st);
    } else {
      launch_replace_r(d.n, r, rh, s->sc.p, w, st);
    }
    rr_ref = rr_true;
  }
}

// The same iteration with every per-element operation in float-float
// arithmetic (dd.cuh, dd.cu, the step-form ILU sweep in ilu.cu).  The
// system is scaled by a power of two (exact) so that ||b|| is about 1; the
// float-float correction x_w is folded into the FP64 solution at every
// reliable update, where the FP64 true residual b - A x replaces the
// recursive one.  Attainable accuracy is then set by the FP64 residual, and
// each cycle's float-float work only has to reduce it by kDelta.
int run_bicgstab_dd(pg_solver *s, double tol, int max_iters, int *iters,
                    int *updates, double *bb_out) {
  cudaStream_t st = stream();
  const SolverDev d = s->dev();
  const RedWork w = s->red();
  const int n = d.n;
  const bool ilu = s->cfg.precond == PG_PREC_ILU0;
  const float2 *jd = s->cfg.precond == PG_PREC_JACOBI ? s->jdinv_dd.p : nullptr;
  float2 *const val = s->pvals_dd.p;
  float2 *const x = s->xd.p, *const r = s->rd.p, *const rh = s->rhd.p;
  float2 *const p = s->pd.p, *const v = s->vd.p, *const ph = s->phd.p;
  float2 *const ss = s->sd.p, *const sh = s->shd.p, *const t = s->td.p;
  const CoarseDev cdev = s->coarse();
  SolverDev d0 = d;  // the deflated form's sweep needs no subdomain sums
  d0.csum = nullptr;
  SolverDev d3 = d0;
  d3.def_y = cdev.y_dd;
  auto precond = [&](int mode, float2 *pv, float2 *z) {
    if (cdev.K && s->cfg.coarse == 2) {
      // A-DEF1 in float-float
      launch_def_pre_dd(cdev, mode, r, pv, v, s->sc.p, st);
      launch_def_in_dd(cdev, n, pv, cdev.tmp_dd, s->sc.p, st);
      kt_mark(s, PG_KT_COARSE, st);
      if (ilu && launch_ilu0_apply_def_dd(d3, cdev.tmp_dd, z, s->sc.p, st)) {
        kt_mark(s, PG_KT_SWEEP, st);
        return;
      }
      if (ilu)
        launch_ilu0_apply_dd(0, d0, r, cdev.tmp_dd, v, z, s->sc.p, st);
      else
        launch_dd_diag_apply(0, n, jd, r, cdev.tmp_dd, v, z, s->sc.p, st);
      kt_mark(s, PG_KT_SWEEP, st);
      launch_coarse_add_dd(cdev, z, s->sc.p, st);
      kt_mark(s, PG_KT_COARSE, st);
      return;
    }
    if (ilu)
      launch_ilu0_apply_dd(mode, d, r, pv, v, z, s->sc.p, st);
    else
      launch_dd_diag_apply(mode, n, jd, r, pv, v, z, s->sc.p, st);
    kt_mark(s, PG_KT_SWEEP, st);
    if (cdev.K) {
      launch_coarse_apply_dd(cdev, pv, z, ilu && d.dd_stream, s->sc.p, st);
      kt_mark(s, PG_KT_COARSE, st);
    }
  };
  auto chunk = [&]() {
    kt_mark(s, -1, st);
    for (int c = 0; c < kChunk; ++c) {
      precond(1, p, ph);
      launch_dd_spmv_v(d, val, ph, v, rh, s->sc.p, w, st);
      kt_mark(s, PG_KT_SPMV, st);
      precond(2, ss, sh);
      launch_dd_spmv_t(d, val, sh, t, ss, s->sc.p, w, st);
      kt_mark(s, PG_KT_SPMV, st);
      launch_dd_update(n, x, r, ph, sh, ss, t, rh, s->sc.p, w, st);
      kt_mark(s, PG_KT_UPDATE, st);
    }
  };
  auto read_scalars = [&]() -> int {
    PG_CUDA(cudaMemcpyAsync(s->sc_host, s->sc.p, sizeof(KScalars),
                            cudaMemcpyDeviceToHost, st));
    PG_CUDA(cudaStreamSynchronize(st));
    return PG_OK;
  };
  KScalars init{};
  init.tol2 = tol * tol;
  init.max_iter = max_iters;
  *s->sc_host = init;
  PG_CUDA(cudaMemcpyAsync(s->sc.p, s->sc_host, sizeof(KScalars),
                          cudaMemcpyHostToDevice, st));
  launch_true_residual(d, s->pvals.p, s->b.p, nullptr, nullptr, s->sc.p, w, st);
  int rc = read_scalars();
  if (rc) return rc;
  const double bb = s->sc_host->rr_true;
  *bb_out = bb;  // unscaled ||b||^2 for the caller's final check
  *iters = 0;
  *updates = 0;
  if (!std::isfinite(bb)) return PG_NON_FINITE;
  if (bb == 0.) {
    PG_CUDA(cudaMemsetAsync(s->x.p, 0, n * sizeof(double), st));
    return PG_OK;
  }
  // power-of-two scale: ||b|| * scale in [0.5, 1)
  const double scale = std::ldexp(1.0, -std::ilogb(std::sqrt(bb)) - 1);
  init.bb = bb * scale * scale;
  init.rr_true = bb;
  *s->sc_host = init;
  PG_CUDA(cudaMemcpyAsync(s->sc.p, s->sc_host, sizeof(KScalars),
                          cudaMemcpyHostToDevice, st));
  PG_CUDA(cudaMemsetAsync(x, 0, n * sizeof(float2), st));
  launch_true_residual(d, s->pvals.p, s->b.p, s->x.p, s->r.p, s->sc.p, w, st);
  launch_dd_set_r(n, s->r.p, scale, r, rh, p, v, true, s->sc.p, w, st);
  if ((rc = read_scalars())) return rc;
  if (s->sc_host->status == PG_NON_FINITE) return PG_NON_FINITE;
  if (s->sc_host->rr_true <= init.tol2 * bb) return PG_OK;
  double rr_ref = s->sc_host->rr_true;
  // progress watch: the true residual norm must fall 10x within
  // kDdStallIters iterations (checked at least that often)
  double prog_rr = rr_ref;
  int prog_it = 0, last_update = 0;
  int restarts = 0;
  bool direct_done = false;
  for (;;) {
    const int slot = cdev.K ? (s->ac_ready ? 5 : 1) : 3;
    if ((rc = run_chunk(s->chunk_graph[slot], s->chunk_launches[slot],
                        direct_done, chunk, s->kt.on)))
      return rc;
    if ((rc = read_scalars())) return rc;
    const KScalars k = *s->sc_host;
    *iters = k.iter;
    if (trace_enabled())
      std::fprintf(stderr,
                   "pg_solver(dd): it %d rr/bb %.3e rho %.3e alpha %.3e omega "
                   "%.3e status %d done %d\n",
                   k.iter, k.rr / init.bb, k.rho, k.alpha, k.omega, k.status,
                   k.done);
    if (k.status == PG_NON_FINITE) return PG_NON_FINITE;
    if (!k.done && !(k.rr < kDelta2 * rr_ref * scale * scale) &&
        k.iter - last_update < kDdStallIters)
      continue;
    last_update = k.iter;
    // reliable update: x += x_w, r = b - A x in FP64
    launch_dd_fold(n, s->x.p, x, 1.0 / scale, st);
    launch_true_residual(d, s->pvals.p, s->b.p, s->x.p, s->r.p, s->sc.p, w, st);
    if ((rc = read_scalars())) return rc;
    const double rr_true = s->sc_host->rr_true;
    ++*updates;
    if (trace_enabled())
      std::fprintf(stderr, "pg_solver(dd): it %d true rr/bb %.3e\n", k.iter,
                   rr_true / bb);
    if (!std::isfinite(rr_true)) return PG_NON_FINITE;
    if (rr_true <= init.tol2 * bb) return PG_OK;
    if (k.iter >= max_iters) return PG_MAX_ITERS;
    const bool restart = k.status == PG_BREAKDOWN;
    if (rr_true < 1e-2 * prog_rr) {
      prog_rr = rr_true;
      prog_it = k.iter;
    }
    // stalled or breaking down in float-float: the FP64 solver carries on
    // from the FP64 iterate
    if (k.iter - prog_it >= kDdStallIters ||
        (restart && ++restarts > kDdMaxRestarts))
      return kDdStalled;
    launch_dd_set_r(n, s->r.p, scale, r, rh, p, v, restart, s->sc.p, w, st);
    rr_ref = rr_true;
  }
}

// z = M^-1 in for the FP64 preconditioner (permuted order): the Schwarz
// ILU(0) sweeps or Jacobi, with the coarse correction of the solver's
// configuration.  in is only read.
int apply_m64(pg_solver *s, const double *in, double *z) {
  cudaStream_t st = stream();
  const SolverDev d = s->dev();
  double *pin = const_cast<double *>(in);  // mode 0 reads it only
  if (s->coarse_on && s->coarse_use && s->cfg.coarse == 2) {
    const CoarseDev c = s->coarse();
    SolverDev d0 = d;
    d0.csum = nullptr;
    launch_def_pre(c, 0, nullptr, pin, nullptr, nullptr, st);
    launch_def_in(c, d.n, pin, c.tmp, nullptr, st);
    SolverDev d3 = d0;
    d3.def_y = c.y;
    if (!(s->cfg.precond == PG_PREC_ILU0 &&
          launch_ilu0_apply_def(d3, c.tmp, z, nullptr, st))) {
      launch_precond<double, double>(s->cfg.precond, 0, d0, s->jdinv.p,
                                     nullptr, c.tmp, nullptr, z, nullptr, st);
      launch_coarse_add(c, z, nullptr, st);
    }
  } else {
    SolverDev d1 = d;
    if (!(s->coarse_on && s->coarse_use)) d1.csum = nullptr;
    launch_precond<double, double>(s->cfg.precond, 0, d1, s->jdinv.p, nullptr,
                                   pin, nullptr, z, nullptr, st);
    if (s->coarse_on && s->coarse_use)
      launch_coarse_apply(s->coarse(), pin, z,
                          s->cfg.precond == PG_PREC_ILU0 &&
                              (d.smem64 > 0 || d.n_lgrp > 0),
                          nullptr, st);
  }
  PG_CUDA(cudaGetLastError());
  return PG_OK;
}

// <a, b> in FP64 with a fixed reduction order, read back to the host
int dot64(pg_solver *s, const double *a, const double *b, double *out) {
  cudaStream_t st = stream();
  launch_mdot((int)s->a.n, 1, a, s->a.n, b, s->kpart.p, s->kdot.p, st);
  PG_CUDA(cudaMemcpyAsync(out, s->kdot.p, sizeof(double),
                          cudaMemcpyDeviceToHost, st));
  PG_CUDA(cudaStreamSynchronize(st));
  return PG_OK;
}

int krylov_buffers(pg_solver *s, int basis) {
  const size_t n = s->a.n;
  for (DevBuf<double> *bf : {&s->k1, &s->k2, &s->k3})
    PG_CUDA(bf->reserve(n));
  const int kmax = basis > 0 ? basis : 1;
  PG_CUDA(s->kpart.reserve((size_t)kmax * 64));
  PG_CUDA(s->kdot.reserve(kmax));
  if (basis > 0) PG_CUDA(s->kV.reserve((size_t)basis * n));
  return PG_OK;
}

// r = b - A x; returns ||r||^2 (and ||b||^2 in *bb when asked)
int true_res64(pg_solver *s, double *r, double *rr) {
  cudaStream_t st = stream();
  const SolverDev d = s->dev();
  launch_spmv_plain(d, s->pvals.p, s->x.p, r, st);
  launch_lincomb(d.n, 1.0, s->b.p, -1.0, r, r, st);
  return dot64(s, r, r, rr);
}

// TFQMR (Freund, SIAM J. Sci. Comput. 14, 1993; Saad, Iterative Methods
// for Sparse Linear Systems, 2nd ed., Alg. 7.8) right-preconditioned as
// Belos "TFQMR" with the Ifpack2 preconditioner: the iteration runs on
// A M^-1 and x advances by M^-1 d, carried as dh.  One iteration here is
// two of the algorithm's half-steps (two products with A M^-1, as one
// BiCGStab iteration).  Stops when the bound sqrt(m+1) tau reaches the
// tolerance and the true residual b - A x confirms it.
int run_tfqmr(pg_solver *s, double tol, int max_iters, int *iters,
              double *bb_out) {
  cudaStream_t st = stream();
  const SolverDev d = s->dev();
  const int n = d.n;
  int rc = krylov_buffers(s, 0);
  if (rc) return rc;
  double *const x = s->x.p, *const w = s->r.p, *const u = s->rh.p;
  double *const uh = s->p.p, *const Bu = s->v.p, *const u1 = s->ph.p;
  double *const uh1 = s->s.p, *const Bu1 = s->sh.p, *const v = s->t.p;
  double *const dh = s->k1.p, *const rstar = s->k2.p, *const tmp = s->k3.p;
  double bb = 0., rr = 0.;
  if ((rc = dot64(s, s->b.p, s->b.p, &bb))) return rc;
  *bb_out = bb;
  *iters = 0;
  if (!std::isfinite(bb)) return PG_NON_FINITE;
  if (bb == 0.) {
    PG_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), st));
    return PG_OK;
  }
  const double bnorm = std::sqrt(bb);
  int restarts = 0;
  for (;;) {  // (re)start from the current x
    if ((rc = true_res64(s, w, &rr))) return rc;
    if (!std::isfinite(rr)) return PG_NON_FINITE;
    if (std::sqrt(rr) <= tol * bnorm) return PG_OK;
    if (*iters >= max_iters) return PG_MAX_ITERS;
    PG_CUDA(cudaMemcpyAsync(u, w, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    PG_CUDA(cudaMemcpyAsync(rstar, w, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    PG_CUDA(cudaMemsetAsync(dh, 0, n * sizeof(double), st));
    if ((rc = apply_m64(s, u, uh))) return rc;
    launch_spmv_plain(d, s->pvals.p, uh, Bu, st);
    PG_CUDA(cudaMemcpyAsync(v, Bu, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    double tau = std::sqrt(rr), theta = 0., eta = 0., rho = rr, alpha = 0.;
    int m = 0;
    bool restart = false;
    // one half-step: w -= alpha Bu_m; dh = uh_m + (theta^2 / alpha) eta dh;
    // x += eta dh; returns 1 when the bound says converged
    auto half = [&](const double *uh_m, const double *Bu_m, int *done) -> int {
      launch_lincomb(n, 1.0, w, -alpha, Bu_m, w, st);
      launch_lincomb(n, 1.0, uh_m, theta * theta / alpha * eta, dh, dh, st);
      double ww = 0.;
      int r2 = dot64(s, w, w, &ww);
      if (r2) return r2;
      theta = std::sqrt(ww) / tau;
      const double c = 1.0 / std::sqrt(1.0 + theta * theta);
      tau = tau * theta * c;
      eta = c * c * alpha;
      launch_lincomb(n, 1.0, x, eta, dh, x, st);
      ++m;
      *done = tau * std::sqrt((double)m + 1.0) <= tol * bnorm;
      return PG_OK;
    };
    while (*iters < max_iters) {
      double sigma = 0.;
      if ((rc = dot64(s, v, rstar, &sigma))) return rc;
      if (sigma == 0. || rho == 0. || !std::isfinite(sigma)) {
        restart = true;
        break;
      }
      alpha = rho / sigma;
      launch_lincomb(n, 1.0, u, -alpha, v, u1, st);          // u_{m+1}
      int done = 0;
      if ((rc = half(uh, Bu, &done))) return rc;             // even m
      if ((rc = apply_m64(s, u1, uh1))) return rc;
      launch_spmv_plain(d, s->pvals.p, uh1, Bu1, st);
      if (!done && (rc = half(uh1, Bu1, &done))) return rc;  // odd m
      ++*iters;
      if (done) break;
      double rho_new = 0.;
      if ((rc = dot64(s, w, rstar, &rho_new))) return rc;
      const double beta = rho_new / rho;
      rho = rho_new;
      launch_lincomb(n, 1.0, w, beta, u1, u, st);            // u = w + beta u1
      if ((rc = apply_m64(s, u, uh))) return rc;
      launch_spmv_plain(d, s->pvals.p, uh, tmp, st);         // A M^-1 u
      // v = A M^-1 u + beta (Bu1 + beta v)
      launch_lincomb(n, 1.0, Bu1, beta, v, v, st);
      launch_lincomb(n, 1.0, tmp, beta, v, v, st);
      PG_CUDA(cudaMemcpyAsync(Bu, tmp, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
      if (!std::isfinite(tau)) return PG_NON_FINITE;
    }
    if (restart && ++restarts > kMaxRestarts) return PG_BREAKDOWN;
    // converged by the bound, breakdown or out of iterations: the true
    // residual decides at the top of the loop
    if (!restart && *iters >= max_iters) {
      if ((rc = true_res64(s, w, &rr))) return rc;
      return std::sqrt(rr) <= tol * bnorm ? PG_OK : PG_MAX_ITERS;
    }
  }
}

// Restarted GMRES (Saad & Schultz, SIAM J. Sci. Stat. Comput. 7, 1986)
// right-preconditioned as Belos "GMRES": restart length `dim` (Belos' "Num
// Blocks"), classical Gram-Schmidt applied twice for the orthogonalisation
// (the dot products of a step in one kernel), Givens rotations on the
// host, x += M^-1 (V y) at the end of every cycle; convergence is the
// implicit residual |g_{j+1}| confirmed by the true residual.
int run_gmres(pg_solver *s, double tol, int max_iters, int dim, int *iters,
              int *cycles, double *bb_out) {
  cudaStream_t st = stream();
  const SolverDev d = s->dev();
  const int n = d.n;
  int rc = krylov_buffers(s, dim + 1);
  if (rc) return rc;
  double *const x = s->x.p, *const r = s->r.p, *const z = s->ph.p;
  double *const w = s->t.p, *const hd = s->kdot.p;
  double *const V = s->kV.p;
  double bb = 0., rr = 0.;
  if ((rc = dot64(s, s->b.p, s->b.p, &bb))) return rc;
  *bb_out = bb;
  *iters = 0;
  *cycles = 0;
  if (!std::isfinite(bb)) return PG_NON_FINITE;
  if (bb == 0.) {
    PG_CUDA(cudaMemsetAsync(x, 0, n * sizeof(double), st));
    return PG_OK;
  }
  const double bnorm = std::sqrt(bb);
  std::vector<double> H((size_t)(dim + 1) * dim, 0.), cs(dim), sn(dim),
      g(dim + 1), h(dim + 1), h2(dim + 1), y(dim);
  for (;;) {
    if ((rc = true_res64(s, r, &rr))) return rc;
    if (!std::isfinite(rr)) return PG_NON_FINITE;
    const double beta = std::sqrt(rr);
    if (beta <= tol * bnorm) return PG_OK;
    if (*iters >= max_iters) return PG_MAX_ITERS;
    ++*cycles;
    launch_lincomb(n, 1.0 / beta, r, 0.0, nullptr, V, st);
    std::fill(g.begin(), g.end(), 0.);
    g[0] = beta;
    int j = 0;
    for (; j < dim && *iters < max_iters; ++j) {
      double *vj = V + (size_t)j * n;
      if ((rc = apply_m64(s, vj, z))) return rc;
      launch_spmv_plain(d, s->pvals.p, z, w, st);
      // two passes of classical Gram-Schmidt against v_0 .. v_j
      for (int pass = 0; pass < 2; ++pass) {
        launch_mdot(n, j + 1, V, n, w, s->kpart.p, hd, st);
        PG_CUDA(cudaMemcpyAsync(pass ? h2.data() : h.data(), hd,
                                (j + 1) * sizeof(double),
                                cudaMemcpyDeviceToHost, st));
        launch_vsub(n, j + 1, V, n, hd, w, st);
      }
      double ww = 0.;
      if ((rc = dot64(s, w, w, &ww))) return rc;  // also waits for h, h2
      for (int i = 0; i <= j; ++i) h[i] += h2[i];
      h[j + 1] = std::sqrt(ww);
      ++*iters;
      if (!std::isfinite(h[j + 1])) return PG_NON_FINITE;
      if (h[j + 1] > 0.)
        launch_lincomb(n, 1.0 / h[j + 1], w, 0.0, nullptr, V + (size_t)(j + 1) * n, st);
      // apply the previous rotations to the new column, then its own
      for (int i = 0; i < j; ++i) {
        const double t = cs[i] * h[i] + sn[i] * h[i + 1];
        h[i + 1] = -sn[i] * h[i] + cs[i] * h[i + 1];
        h[i] = t;
      }
      const double den = std::hypot(h[j], h[j + 1]);
      cs[j] = den > 0. ? h[j] / den : 1.;
      sn[j] = den > 0. ? h[j + 1] / den : 0.;
      h[j] = den;
      h[j + 1] = 0.;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      for (int i = 0; i <= j; ++i) H[(size_t)i * dim + j] = h[i];
      if (std::fabs(g[j + 1]) <= tol * bnorm || den == 0.) {
        ++j;
        break;
      }
    }
    // y = H^-1 g (upper triangular, j columns); x += M^-1 (V y)
    for (int i = j - 1; i >= 0; --i) {
      double acc = g[i];
      for (int k = i + 1; k < j; ++k) acc -= H[(size_t)i * dim + k] * y[k];
      const double hii = H[(size_t)i * dim + i];
      y[i] = hii != 0. ? acc / hii : 0.;
    }
    PG_CUDA(cudaMemsetAsync(w, 0, n * sizeof(double), st));
    // w = V y, as w -= V (-y)
    for (int i = 0; i < j; ++i) y[i] = -y[i];
    PG_CUDA(cudaMemcpyAsync(hd, y.data(), j * sizeof(double),
                            cudaMemcpyHostToDevice, st));
    launch_vsub(n, j, V, n, hd, w, st);
    if ((rc = apply_m64(s, w, z))) return rc;
    launch_lincomb(n, 1.0, x, 1.0, z, x, st);
    PG_CUDA(cudaStreamSynchronize(st));
  }
}

bool use_dd(const pg_solver *s) {
  const SolverDev d = s->dev();
  return s->cfg.precision == PG_MIXED &&
         (s->cfg.precond != PG_PREC_ILU0 || d.smem_dd > 0 ||
          (d.smem64 > 0 && d.srec_dds));
}

// The mixed solver's ILU(0) sweep has two record forms: warp-wide steps
// (few instructions per level, but every step padded to 32 rows) and the
// level blobs of the FP64 stream (compact).  Which is faster depends on the
// level widths of the mesh, so the first factorisation after an analysis
// times three applications of each and keeps the faster.
int choose_dd_sweep(pg_solver *s) {
  const SolverDev d0 = s->dev();
  const bool has_steps = d0.smem_dd > 0, has_blobs = d0.smem64 > 0 && d0.srec_dds;
  if (d0.n_lgrp32 > 0) {  // mixed_sweep 3: FP32-weight line form
    s->dd_stream = 1;
    return PG_OK;
  }
  if (has_steps && s->cfg.mixed_sweep == 1) {
    s->dd_stream = 0;
    return PG_OK;
  }
  if (has_blobs && s->cfg.mixed_sweep == 2) {
    s->dd_stream = 1;
    return PG_OK;
  }
  if (!has_steps || !has_blobs) {
    s->dd_stream = has_blobs ? 1 : 0;
    return PG_OK;
  }
  cudaStream_t st = stream();
  const int64_t n = s->a.n;
  PG_CUDA(cudaMemsetAsync(s->pd.p, 0, n * sizeof(float2), st));
  float best = 1e30f;
  int pick = 0;
  cudaEvent_t e0 = nullptr, e1 = nullptr;  // the solve's own events stay put
  PG_CUDA(cudaEventCreate(&e0));
  cudaError_t ce = cudaEventCreate(&e1);
  for (int form = 0; form < 2 && ce == cudaSuccess; ++form) {
    s->dd_stream = form;
    const SolverDev d = s->dev();
    launch_ilu0_apply_dd(0, d, nullptr, s->pd.p, nullptr, s->phd.p, nullptr, st);
    ce = cudaEventRecord(e0, st);
    for (int k = 0; k < 3; ++k)
      launch_ilu0_apply_dd(0, d, nullptr, s->pd.p, nullptr, s->phd.p, nullptr, st);
    if (ce == cudaSuccess) ce = cudaEventRecord(e1, st);
    if (ce == cudaSuccess) ce = cudaEventSynchronize(e1);
    if (ce == cudaSuccess) ce = cudaGetLastError();
    float ms = 0.f;
    if (ce == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) {
      best = ms;
      pick = form;
    }
  }
  cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  PG_CUDA(ce);
  s->dd_stream = pick;
  s->drop_graphs();  // the chunk graph holds the apply kernel
  return PG_OK;
}

int factor(pg_solver *s, cudaStream_t st) {
  const SolverDev d = s->dev();
  const bool dd = use_dd(s);
  if (s->cfg.precond == PG_PREC_ILU0) {
    PG_CUDA(cudaMemsetAsync(s->bad.p, 0, sizeof(int), st));
    launch_ilu0_factor(d, s->pvals.p, s->bad.p, dd, st);
    if (s->coarse_on) {
      // beside the ILU(0) factorisation and the first iterations; with
      // cfg.coarse_warm = -2 into the buffer the next solve will apply,
      // the current one staying in use, and the A Z values (read by the
      // solve) on the factorisation stream
      const bool reuse = s->cfg.coarse_warm == -2;
      if (reuse) {
        int rj = join_coarse(s);  // the previous inverse becomes current
        if (rj) return rj;
      }
      const int target = reuse && s->ac_valid ? 1 - s->ac_ready : s->ac_ready;
      const bool use = s->coarse_use;
      s->coarse_use = true;
      CoarseDev ct = s->coarse();
      ct.ac = s->ac_buf(target);
      cudaStream_t azs = reuse ? st : s->side2;
      if (reuse && s->cfg.coarse == 2) {
        launch_az_values(ct, (int)s->a.n, s->prp.p, s->pvals.p, azs);
        if (dd)
          launch_dd_split((int64_t)s->a.azj.size(), s->c_azv.p, 1.0,
                          s->c_azv_dd.p, azs);
      }
      PG_CUDA(cudaEventRecord(s->ev_cvals, st));
      PG_CUDA(cudaStreamWaitEvent(s->side2, s->ev_cvals, 0));
      if (s->c_lu) {
        int rc = launch_coarse_setup_lu(ct, s->c_lu, s->c_vals.p, s->pvals.p,
                                        s->prp.p, s->gj_graph_of(target),
                                        s->side2);
        if (rc) return rc;
      } else {
        launch_coarse_setup(ct, s->pvals.p, s->prp.p, s->gj_graph_of(target),
                            s->side2);
      }
      if (!reuse && s->cfg.coarse == 2) {
        launch_az_values(ct, (int)s->a.n, s->prp.p, s->pvals.p, azs);
        if (dd)
          launch_dd_split((int64_t)s->a.azj.size(), s->c_azv.p, 1.0,
                          s->c_azv_dd.p, azs);
      }
      s->coarse_use = use;
      PG_CUDA(cudaEventRecord(s->ev_coarse, s->side2));
      s->coarse_pending = true;
      s->ac_next = target;
    }
  } else if (s->cfg.precond == PG_PREC_JACOBI) {
    launch_jacobi_diag(d, s->pvals.p, s->jdinv.p, st);
    if (dd) launch_dd_split(d.n, s->jdinv.p, 1.0, s->jdinv_dd.p, st);
  }
  if (dd) launch_dd_split(d.nnz, s->pvals.p, 1.0, s->pvals_dd.p, st);
  PG_CUDA(cudaGetLastError());
  if (dd && s->cfg.precond == PG_PREC_ILU0 && s->dd_stream < 0)
    return choose_dd_sweep(s);  // library stream only (see start_factor)
  return PG_OK;
}

// After a value hand-over: factor on the side stream, so the work the
// caller issues next on the library stream (an initial-guess inference, a
// right-hand side) overlaps it.  The first factorisation of a mixed solver
// times its sweep forms and stays on the library stream.
int start_factor(pg_solver *s) {
  if (use_dd(s) && s->cfg.precond == PG_PREC_ILU0 && s->dd_stream < 0)
    return PG_OK;
  PG_CUDA(cudaEventRecord(s->ev_vals, stream()));
  PG_CUDA(cudaStreamWaitEvent(s->side, s->ev_vals, 0));
  int rc = factor(s, s->side);
  if (rc) return rc;
  PG_CUDA(cudaEventRecord(s->ev_fact, s->side));
  s->fact_pending = true;
  return PG_OK;
}

}  // namespace

// ------------------------------------------------------------------ C ABI
extern "C" void pg_solver_default_cfg(pg_solver_cfg *cfg) {
  if (!cfg) return;
  cfg->tolerance = 1e-8;
  cfg->max_iters = 500;
  cfg->precond = PG_PREC_ILU0;
  cfg->subdomain_rows = 0;
  cfg->precision = PG_FP64;
  cfg->mixed_sweep = 0;
  cfg->coarse = 0;
  cfg->coarse_warm = -1;
  cfg->krylov = PG_KRYLOV_BICGSTAB;
  cfg->ilu_fill = 0;
  cfg->krylov_dim = 0;
  cfg->reserved_i = 0;
  cfg->reserved_d = 0.;
}

extern "C" int pg_solver_create(const pg_solver_cfg *cfg, pg_solver **out) {
  PG_CHECK_ARG(out, "pg_solver_create: out is NULL");
  *out = nullptr;
  pg_solver_cfg c;
  pg_solver_default_cfg(&c);
  if (cfg) c = *cfg;
  PG_CHECK_ARG(c.tolerance > 0. && c.max_iters > 0, "pg_solver_create: bad tolerance/max_iters");
  PG_CHECK_ARG(c.precond >= PG_PREC_NONE && c.precond <= PG_PREC_ILU0,
               "pg_solver_create: bad preconditioner");
  PG_CHECK_ARG(c.precision == PG_FP64 || c.precision == PG_MIXED,
               "pg_solver_create: bad precision");
  PG_CHECK_ARG(c.mixed_sweep >= 0 && c.mixed_sweep <= 3,
               "pg_solver_create: bad mixed_sweep");
  PG_CHECK_ARG(c.coarse >= 0 && c.coarse <= 2, "pg_solver_create: bad coarse");
  PG_CHECK_ARG(c.coarse_warm >= -2, "pg_solver_create: bad coarse_warm");
  PG_CHECK_ARG(c.krylov >= PG_KRYLOV_BICGSTAB && c.krylov <= PG_KRYLOV_GMRES,
               "pg_solver_create: bad krylov");
  PG_CHECK_ARG(c.krylov == PG_KRYLOV_BICGSTAB || c.precision == PG_FP64,
               "pg_solver_create: TFQMR and GMRES run in FP64");
  PG_CHECK_ARG(c.ilu_fill >= 0 && c.ilu_fill <= 8,
               "pg_solver_create: ilu_fill must be 0 .. 8");
  PG_CHECK_ARG(c.krylov_dim >= 0, "pg_solver_create: bad krylov_dim");
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0 || !stream()) {
    set_error("no CUDA device available: libphase_gb300 has no CPU path");
    return PG_CUDA_ERROR;
  }
  auto *s = new (std::nothrow) pg_solver();
  PG_CHECK_ARG(s, "pg_solver_create: out of host memory");
  s->cfg = c;
  int rc = ensure_host_state(s);
  if (rc) {
    delete s;
    return rc;
  }
  *out = s;
  return PG_OK;
}

extern "C" int pg_solver_destroy(pg_solver *s) {
  if (s) cudaStreamSynchronize(stream());
  delete s;
  return PG_OK;
}

extern "C" int pg_solver_set_rank(pg_solver *s, int64_t n) {
  PG_CHECK_ARG(s && n > 0, "pg_solver_set_rank: bad argument");
  PG_CHECK_ARG(n < ((int64_t)1 << 31), "pg_solver_set_rank: rank too large");
  if (s->rank != n) {
    s->analysed = false;
    s->have_x = false;
  }
  s->rank = n;
  return PG_OK;
}

extern "C" int pg_solver_set_row_coords(pg_solver *s, const double *xy) {
  PG_CHECK_ARG(s, "pg_solver_set_row_coords: NULL solver");
  std::vector<double> nx, ny;
  if (xy) {
    PG_CHECK_ARG(s->rank > 0, "pg_solver_set_row_coords: set_rank first");
    nx.resize(s->rank);
    ny.resize(s->rank);
    for (int64_t i = 0; i < s->rank; ++i) {
      nx[i] = xy[2 * i];
      ny[i] = xy[2 * i + 1];
    }
  }
  if (nx == s->row_x && ny == s->row_y) return PG_OK;  // unchanged
  s->row_x.swap(nx);
  s->row_y.swap(ny);
  s->analysed = false;  // the next set_csr re-cuts the subdomains
  return PG_OK;
}

extern "C" int pg_solver_set_csr(pg_solver *s, const int32_t *row_ptr,
                                 const int32_t *col_ind, const double *vals,
                                 int ptr_kind) {
  PG_CHECK_ARG(s && row_ptr && col_ind && vals, "pg_solver_set_csr: NULL arg");
  PG_CHECK_ARG(s->rank > 0, "pg_solver_set_csr: set_rank first");
  const int64_t n = s->rank;
  cudaStream_t st = stream();
  // host copies of the pattern are needed for (re)analysis
  std::vector<int32_t> h_rp, h_ci;
  const int32_t *hrp = row_ptr, *hci = col_ind;
  int64_t n_src;
  if (ptr_kind == PG_DEVICE) {
    int32_t last = 0;
    PG_CUDA(cudaMemcpyAsync(&last, row_ptr + n, sizeof(int32_t),
                            cudaMemcpyDeviceToHost, st));
    PG_CUDA(cudaStreamSynchronize(st));
    n_src = last;
  } else {
    n_src = row_ptr[n];
  }
  PG_CHECK_ARG(n_src >= 0, "pg_solver_set_csr: bad row_ptr");
  // stage pattern + values on the device
  const int32_t *drp = row_ptr, *dci = col_ind;
  const double *dv = vals;
  if (ptr_kind != PG_DEVICE) {
    PG_CUDA(s->st_rp.upload(row_ptr, n + 1));
    PG_CUDA(s->st_ci.upload(col_ind, n_src));
    PG_CUDA(s->st_vals.upload(vals, n_src));
    drp = s->st_rp.p;
    dci = s->st_ci.p;
    dv = s->st_vals.p;
  }
  bool same = s->analysed && s->eqn_pattern == 0 && s->a.n == n &&
              s->a.n_src == n_src;
  if (same) {
    *s->diff_host = 0;
    PG_CUDA(cudaMemsetAsync(s->diff.p, 0, sizeof(unsigned), st));
    k_count_diff<<<grid_for(n + 1), 256, 0, st>>>(n + 1, drp, s->raw_rp.p, s->diff.p);
    count_launches(1);
    k_count_diff<<<grid_for(n_src), 256, 0, st>>>(n_src, dci, s->raw_ci.p, s->diff.p);
    count_launches(1);
    PG_CUDA(cudaMemcpyAsync(s->diff_host, s->diff.p, sizeof(unsigned),
                            cudaMemcpyDeviceToHost, st));
    PG_CUDA(cudaStreamSynchronize(st));
    same = *s->diff_host == 0;
  }
  if (!same) {
    if (ptr_kind == PG_DEVICE) {
      h_rp.resize(n + 1);
      h_ci.resize(n_src);
      PG_CUDA(cudaMemcpyAsync(h_rp.data(), row_ptr, (n + 1) * 4,
                              cudaMemcpyDeviceToHost, st));
      PG_CUDA(cudaMemcpyAsync(h_ci.data(), col_ind, n_src * 4,
                              cudaMemcpyDeviceToHost, st));
      PG_CUDA(cudaStreamSynchronize(st));
      hrp = h_rp.data();
      hci = h_ci.data();
    }
    const bool xy = (int64_t)s->row_x.size() == n;
    int rc = analyse(n, hrp, hci, subdomain_rows_for(s->cfg, n), s->a,
                     nullptr, xy ? s->row_x.data() : nullptr,
                     xy ? s->row_y.data() : nullptr, ilu_fill_of(s->cfg));
    if (rc) return rc;
    rc = upload_analysis(s);
    if (rc) return rc;
    PG_CUDA(s->raw_rp.upload(hrp, n + 1));
    PG_CUDA(s->raw_ci.upload(hci, n_src));
    s->eqn_pattern = 0;
  }
  int rj = join_factor(s);  // a pending factorisation still reads pvals
  if (!rj) rj = join_coarse(s);
  if (rj) return rj;
  launch_permute_values((int)s->a.nnz, s->psrc.p, dv, s->pvals.p,
                        (int)s->a.dup_dst.size(), s->dup_dst.p, s->dup_src.p, st);
  if (s->sell_on)
    launch_sell_values((int64_t)s->a.sell_col.size(), s->sell_src.p, s->pvals.p,
                       s->sell_val.p, st);
  PG_CUDA(cudaGetLastError());
  s->have_vals = true;
  s->factored = false;
  s->eqn_src = nullptr;  // the values no longer come from a device equation
  return start_factor(s);
}

// The matrix of a device equation and its right-hand side `component`
// (0, or 1 for the y rows of a momentum equation, whose two components
// share one matrix).  With reuse, a call with the same equation at the
// same assembly as the previous one only replaces the right-hand side: the
// values, the factorisation and the coarse inverse are kept.
static int set_eqn(pg_solver *s, const pg_eqn *e, int component, bool reuse) {
  cudaStream_t st = stream();
  const double *rhs = e->rhs.p + (size_t)component * e->p.n;
  if (reuse && s->eqn_src == e && s->eqn_version == e->version && s->analysed &&
      s->eqn_pattern == e->pattern_id && s->rank == e->p.n) {
    int rj = join_factor(s);  // the solve's own rhs buffer is reused
    if (rj) return rj;
    launch_permute_vec((int)s->a.n, s->perm.p, rhs, -1.0, s->b.p, st);
    PG_CUDA(cudaGetLastError());
    s->have_rhs = true;
    return PG_OK;
  }
  if (s->rank != e->p.n) {
    s->rank = e->p.n;
    s->analysed = false;
  }
  if (!s->analysed || s->eqn_pattern != e->pattern_id) {
    // rows are cells: cut the Schwarz subdomains by the cell centres
    const pg::HostMesh &hm = e->mesh->h;
    const bool xy = e->p.n == hm.n_cells;
    int rc = analyse(e->p.n, e->p.row_ptr.data(), e->p.col_ind.data(),
                     subdomain_rows_for(s->cfg, e->p.n), s->a,
                     nullptr, xy ? hm.cx.data() : nullptr,
                     xy ? hm.cy.data() : nullptr, ilu_fill_of(s->cfg));
    if (rc) return rc;
    rc = upload_analysis(s);
    if (rc) return rc;
    s->eqn_pattern = e->pattern_id;
  }
  int rj = join_factor(s);  // a pending factorisation still reads pvals
  if (!rj) rj = join_coarse(s);
  if (rj) return rj;
  launch_permute_values((int)s->a.nnz, s->psrc.p, e->vals.p, s->pvals.p,
                        (int)s->a.dup_dst.size(), s->dup_dst.p, s->dup_src.p, st);
  if (s->sell_on)
    launch_sell_values((int64_t)s->a.sell_col.size(), s->sell_src.p, s->pvals.p,
                       s->sell_val.p, st);
  // the solver receives -rhs_ (FiniteVolumeEquation.tpp:73)
  launch_permute_vec((int)s->a.n, s->perm.p, rhs, -1.0, s->b.p, st);
  PG_CUDA(cudaGetLastError());
  s->have_vals = true;
  s->have_rhs = true;
  s->factored = false;
  s->eqn_src = e;
  s->eqn_version = e->version;
  return start_factor(s);
}

extern "C" int pg_solver_set_eqn(pg_solver *s, const pg_eqn *e) {
  PG_CHECK_ARG(s && e, "pg_solver_set_eqn: NULL arg");
  PG_CHECK_ARG(!e->momentum,
               "pg_solver_set_eqn: a momentum equation has two right-hand "
               "sides; use pg_solver_set_eqn_component");
  return set_eqn(s, e, 0, false);
}

extern "C" int pg_solver_set_eqn_component(pg_solver *s, const pg_eqn *e,
                                           int component) {
  PG_CHECK_ARG(s && e, "pg_solver_set_eqn_component: NULL arg");
  PG_CHECK_ARG(component == 0 || (component == 1 && e->momentum),
               "pg_solver_set_eqn_component: component must be 0, or 1 for "
               "a momentum equation");
  return set_eqn(s, e, component, true);
}

extern "C" int pg_solver_set_rhs(pg_solver *s, const double *rhs, int ptr_kind) {
  PG_CHECK_ARG(s && rhs, "pg_solver_set_rhs: NULL arg");
  PG_CHECK_ARG(s->analysed, "pg_solver_set_rhs: set the matrix first");
  const double *d = rhs;
  if (ptr_kind != PG_DEVICE) {
    PG_CUDA(s->st_vec.upload(rhs, s->a.n));
    d = s->st_vec.p;
  }
  launch_permute_vec((int)s->a.n, s->perm.p, d, 1.0, s->b.p, stream());
  PG_CUDA(cudaGetLastError());
  s->have_rhs = true;
  return PG_OK;
}

extern "C" int pg_solver_set_guess(pg_solver *s, const double *x0, int ptr_kind) {
  PG_CHECK_ARG(s, "pg_solver_set_guess: NULL solver");
  PG_CHECK_ARG(s->analysed, "pg_solver_set_guess: set the matrix first");
  if (!x0) {  // zero initial guess
    PG_CUDA(cudaMemsetAsync(s->x.p, 0, s->a.n * sizeof(double), stream()));
    s->have_x = true;
    return PG_OK;
  }
  const double *d = x0;
  if (ptr_kind != PG_DEVICE) {
    PG_CUDA(s->st_vec.upload(x0, s->a.n));
    d = s->st_vec.p;
  }
  launch_permute_vec((int)s->a.n, s->perm.p, d, 1.0, s->x.p, stream());
  PG_CUDA(cudaGetLastError());
  s->have_x = true;
  return PG_OK;
}

extern "C" int pg_solver_solve(pg_solver *s, pg_solve_stats *stats) {
  PG_CHECK_ARG(s, "pg_solver_solve: NULL solver");
  PG_CHECK_ARG(s->analysed && s->have_vals && s->have_rhs,
               "pg_solver_solve: matrix and rhs must be set first");
  cudaStream_t st = stream();
  const int64_t n = s->a.n;
  s->kt.used = 0;
  s->kt.dropped = 0;
  if (!s->have_x) PG_CUDA(cudaMemsetAsync(s->x.p, 0, n * sizeof(double), st));
  PG_CUDA(cudaEventRecord(s->ev[0], st));
  // the factorisation started at the hand-over, or now (unless the values
  // are those of the last factorisation)
  int rc = s->fact_pending ? join_factor(s) : s->factored ? PG_OK : factor(s, st);
  if (rc) return rc;
  s->factored = true;
  PG_CUDA(cudaEventRecord(s->ev[1], st));
  if (s->cfg.precond == PG_PREC_ILU0) {
    PG_CUDA(cudaMemcpyAsync(s->bad_host, s->bad.p, sizeof(int),
                            cudaMemcpyDeviceToHost, st));
  }
  int iters = 0, outer = 0;
  const double tol = s->cfg.tolerance;
  const SolverDev d = s->dev();
  const RedWork w = s->red();
  double bb = 0.;
  int fp64_iters = 0;  // FP64 iterations after a float-float hand-over
  const bool dd = use_dd(s);
  auto run = [&](int max_iters, int *it, int *up) {
    if (s->cfg.krylov == PG_KRYLOV_TFQMR) {
      *up = 0;
      return run_tfqmr(s, tol, max_iters, it, &bb);
    }
    if (s->cfg.krylov == PG_KRYLOV_GMRES)
      return run_gmres(s, tol, max_iters,
                       s->cfg.krylov_dim > 0 ? s->cfg.krylov_dim : 300, it, up,
                       &bb);
    return dd ? run_bicgstab_dd(s, tol, max_iters, it, up, &bb)
              : run_bicgstab(s, tol, max_iters, it, up, &bb);
  };
  int status;
  const int warm = s->cfg.coarse_warm >= 0 ? s->cfg.coarse_warm
                   : s->a.n_sub >= kCoarseStagedK && !s->c_lu ? kCoarseWarmIters
                                                              : 0;
  if (s->coarse_pending && s->cfg.coarse_warm == -2 && s->ac_valid) {
    // the previous factorisation's coarse inverse preconditions the whole
    // solve (a fixed operator) while the new one is built on side2
    status = run(s->cfg.max_iters, &iters, &outer);
  } else if (s->coarse_pending && warm > 0 && s->cfg.max_iters > warm) {
    // while the coarse inverse is built on side2: `warm` one-level
    // iterations, then a restart from their x with the two-level
    // preconditioner (a fixed count, so results do not depend on timing)
    s->coarse_use = false;
    status = run(warm, &iters, &outer);
    s->coarse_use = true;
    if (status == PG_MAX_ITERS || status == kDdStalled || status == PG_BREAKDOWN) {
      int rj = join_coarse(s);
      if (rj) return rj;
      int it2 = 0, up2 = 0;
      status = run(s->cfg.max_iters - iters, &it2, &up2);
      iters += it2;
      outer += up2;
    }
  } else {
    int rj = join_coarse(s);
    if (rj) return rj;
    status = run(s->cfg.max_iters, &iters, &outer);
  }
  if (status == kDdStalled) {
    // FP64 BiCGStab from the float-float solver's (folded FP64) iterate
    int it2 = 0, up2 = 0;
    if (trace_enabled())
      std::fprintf(stderr, "pg_solver(dd): stalled at it %d, FP64 continues\n",
                   iters);
    status = run_bicgstab(s, tol, std::max(s->cfg.max_iters - iters, 1), &it2,
                          &up2, &bb);
    iters += it2;
    outer += up2;
    fp64_iters = it2;
  }
  if (status == PG_CUDA_ERROR) return status;
  // final true residual in FP64 and the solution in the caller's order
  launch_true_residual(d, s->pvals.p, s->b.p, s->x.p, nullptr, s->sc.p, w, st);
  launch_unpermute_vec((int)n, s->perm.p, s->x.p, s->xout.p, st);
  PG_CUDA(cudaGetLastError());
  PG_CUDA(cudaEventRecord(s->ev[2], st));
  PG_CUDA(cudaMemcpyAsync(s->sc_host, s->sc.p, sizeof(KScalars),
                          cudaMemcpyDeviceToHost, st));
  PG_CUDA(cudaStreamSynchronize(st));
  int timed_out = 0;
  if (s->cfg.precond == PG_PREC_ILU0) {
    PG_CUDA(cudaMemcpy(&timed_out, s->err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (timed_out) PG_CUDA(cudaMemsetAsync(s->err.p, 0, sizeof(int), st));
  }
  float ms_fact = 0.f, ms_all = 0.f;
  cudaEventElapsedTime(&ms_fact, s->ev[0], s->ev[1]);
  cudaEventElapsedTime(&ms_all, s->ev[0], s->ev[2]);
  const double rel = bb > 0. ? std::sqrt(s->sc_host->rr_true / bb)
                   : status == PG_NON_FINITE ? NAN : 0.;
  if (s->cfg.precond == PG_PREC_ILU0 && *s->bad_host > 0 && !(rel <= tol))
    status = PG_BREAKDOWN;
  if (status == PG_OK && !(rel <= tol)) status = PG_MAX_ITERS;
  if (!std::isfinite(rel)) status = PG_NON_FINITE;
  if (timed_out) status = PG_TIMEOUT;
  s->have_x = true;  // warm start for the next solve, as Belos reuses x_
  if (stats) {
    stats->iters = iters;
    stats->outer_iters = outer;
    stats->status = status;
    stats->fp64_iters = fp64_iters;
    stats->rel_residual = rel;
    stats->ms = ms_all;
    stats->setup_ms = ms_fact;
  }
  if (status != PG_OK)
    set_error("pg_solver_solve: status " + std::to_string(status) + " after " +
              std::to_string(iters) + " iterations, relative residual " +
              std::to_string(rel));
  return status;
}

extern "C" int pg_solver_get_x(const pg_solver *s, double *x, int ptr_kind) {
  PG_CHECK_ARG(s && x, "pg_solver_get_x: NULL arg");
  PG_CHECK_ARG(s->analysed, "pg_solver_get_x: nothing solved");
  PG_CUDA(copy_out(x, s->xout.p, s->a.n * sizeof(double), ptr_kind));
  PG_CUDA(cudaStreamSynchronize(stream()));
  return PG_OK;
}

extern "C" uint64_t pg_kernel_launches(void) { return launch_count(); }

extern "C" int pg_solver_trace_kernels(pg_solver *s, int on) {
  PG_CHECK_ARG(s, "pg_solver_trace_kernels: NULL solver");
  s->kt.on = on != 0;
  s->kt.used = 0;
  s->kt.dropped = 0;
  return PG_OK;
}

extern "C" int pg_solver_kernel_times(pg_solver *s, double *ms, int64_t *count,
                                      int64_t *dropped) {
  PG_CHECK_ARG(s && ms && count, "pg_solver_kernel_times: bad argument");
  PG_CUDA(cudaStreamSynchronize(stream()));
  for (int k = 0; k < PG_KT_N; ++k) {
    ms[k] = 0.;
    count[k] = 0;
  }
  const auto &t = s->kt;
  for (size_t i = 1; i < t.used; ++i) {
    const int k = t.kind[i];
    if (k < 0 || k >= PG_KT_N) continue;
    float f = 0.f;
    PG_CUDA(cudaEventElapsedTime(&f, t.ev[i - 1], t.ev[i]));
    ms[k] += f;
    ++count[k];
  }
  if (dropped) *dropped = t.dropped;
  return PG_OK;
}

extern "C" int pg_solver_profile(pg_solver *s, int reps, double *ms) {
  PG_CHECK_ARG(s && ms && reps > 0, "pg_solver_profile: bad argument");
  PG_CHECK_ARG(s->analysed && s->have_vals && s->have_x,
               "pg_solver_profile: solve a system first");
  int rj = join_factor(s);
  if (!rj) rj = join_coarse(s);
  if (rj) return rj;
  cudaStream_t st = stream();
  const SolverDev d = s->dev();
  const RedWork w = s->red();
  const int64_t n = s->a.n;
  const int g = grid_for(n);
  const bool dd = use_dd(s);
  // scratch vectors with benign non-zero contents, so no kernel takes its
  // breakdown/convergence exit; the solver's own state is left untouched
  DevBuf<double> d8[8];
  DevBuf<float2> f8[8];
  for (int k = 0; k < 8; ++k) {
    PG_CUDA(d8[k].reserve(n));
    k_fill_profile<<<g, 256, 0, st>>>(n, d8[k].p, nullptr, k);
    if (dd) {
      PG_CUDA(f8[k].reserve(n));
      launch_dd_split(n, d8[k].p, 1.0, f8[k].p, st);
    }
  }
  KScalars k{};
  k.max_iter = 1 << 30;
  k.alpha = k.omega = k.beta = k.rho = k.rho_prev = 1.0;
  k.alpha_dd = k.omega_dd = k.beta_dd = make_float2(1.f, 0.f);
  k.bb = 1.0;
  *s->sc_host = k;
  PG_CUDA(cudaMemcpyAsync(s->sc.p, s->sc_host, sizeof(KScalars),
                          cudaMemcpyHostToDevice, st));
  float t = 0.f;
  auto timed = [&](auto &&launch, double *out) -> int {
    launch();  // warm
    PG_CUDA(cudaEventRecord(s->ev[0], st));
    for (int i = 0; i < reps; ++i) launch();
    PG_CUDA(cudaEventRecord(s->ev[1], st));
    PG_CUDA(cudaEventSynchronize(s->ev[1]));
    PG_CUDA(cudaGetLastError());
    cudaEventElapsedTime(&t, s->ev[0], s->ev[1]);
    *out = (double)t / reps;
    return PG_OK;
  };
  for (int i = 0; i < 9; ++i) ms[i] = 0.;
  // vectors: 0 ph/sh, 1 v/t, 2 rh, 3 r, 4 p/s, 5 x, 6 z
  int rc = timed([&] { launch_spmv_v<double, double>(d, s->pvals.p, d8[0].p, d8[1].p, d8[2].p, s->sc.p, w, st); }, &ms[0]);
  if (!rc) rc = timed([&] { launch_precond<double, double>(s->cfg.precond, 1, d, s->jdinv.p, d8[3].p, d8[4].p, d8[1].p, d8[6].p, s->sc.p, st); }, &ms[1]);
  if (!rc) rc = timed([&] { launch_update<double>(d.n, d8[5].p, d8[3].p, d8[0].p, d8[6].p, d8[4].p, d8[1].p, d8[2].p, s->sc.p, w, st); }, &ms[2]);
  // the coarse matrix and its inverse (into the buffer the solves apply)
  auto coarse_setup = [&] {
    if (s->c_lu)
      launch_coarse_setup_lu(s->coarse(), s->c_lu, s->c_vals.p, s->pvals.p,
                             s->prp.p, s->gj_graph_of(s->ac_ready), st);
    else
      launch_coarse_setup(s->coarse(), s->pvals.p, s->prp.p,
                          s->gj_graph_of(s->ac_ready), st);
  };
  if (!rc && s->cfg.precond == PG_PREC_ILU0)
    rc = timed([&] {
      launch_ilu0_factor(d, s->pvals.p, s->bad.p, dd, st);
      if (s->coarse_on) coarse_setup();
    }, &ms[3]);
  if (!rc && s->coarse_on) rc = timed(coarse_setup, &ms[8]);
  if (!rc && s->coarse_on) {
    const CoarseDev c = s->coarse();
    if (s->cfg.coarse == 2 && dd)
      rc = timed([&] {
        launch_def_pre_dd(c, 1, f8[3].p, f8[4].p, f8[1].p, s->sc.p, st);
        launch_def_in_dd(c, (int)n, f8[4].p, c.tmp_dd, s->sc.p, st);
      }, &ms[7]);
    else if (s->cfg.coarse == 2)
      rc = timed([&] {
        launch_def_pre(c, 1, d8[3].p, d8[4].p, d8[1].p, s->sc.p, st);
        launch_def_in(c, d.n, d8[4].p, c.tmp, s->sc.p, st);
      }, &ms[7]);
    else
      rc = timed([&] { launch_coarse_apply(c, d8[4].p, d8[6].p, true, s->sc.p, st); }, &ms[7]);
  }
  if (!rc && dd) {
    if (s->cfg.precond == PG_PREC_ILU0)
      rc = timed([&] { launch_ilu0_apply_dd(1, d, f8[3].p, f8[4].p, f8[1].p, f8[6].p, s->sc.p, st); }, &ms[4]);
    if (!rc) rc = timed([&] { launch_dd_spmv_v(d, s->pvals_dd.p, f8[0].p, f8[1].p, f8[2].p, s->sc.p, w, st); }, &ms[5]);
    if (!rc) rc = timed([&] { launch_dd_update(d.n, f8[5].p, f8[3].p, f8[0].p, f8[6].p, f8[4].p, f8[1].p, f8[2].p, s->sc.p, w, st); }, &ms[6]);
  }
  PG_CUDA(cudaStreamSynchronize(st));
  return rc;
}

extern "C" int pg_solver_apply_precond(pg_solver *s, const double *r,
                                       double *z, int ptr_kind) {
  PG_CHECK_ARG(s && r && z, "pg_solver_apply_precond: NULL arg");
  PG_CHECK_ARG(s->analysed && s->have_vals,
               "pg_solver_apply_precond: set the matrix first");
  cudaStream_t st = stream();
  const int64_t n = s->a.n;
  int rc = s->fact_pending ? join_factor(s) : factor(s, st);
  if (!rc) rc = join_coarse(s);
  if (rc) return rc;
  s->factored = true;
  const SolverDev d = s->dev();  // after factor(): the sweep form is chosen
  const double *dr = r;
  if (ptr_kind != PG_DEVICE) {
    PG_CUDA(s->st_vec.upload(r, n));
    dr = s->st_vec.p;
  }
  // z = M^-1 r in the permuted order (mode 0 reads p, writes ph)
  launch_permute_vec((int)n, s->perm.p, dr, 1.0, s->p.p, st);
  if (use_dd(s)) {
    launch_dd_split(n, s->p.p, 1.0, s->pd.p, st);
    const bool def = s->coarse_on && s->cfg.coarse == 2;
    const CoarseDev c = s->coarse();
    SolverDev d0 = d;
    d0.csum = def ? nullptr : d.csum;
    float2 *in = s->pd.p;
    bool fused = false;
    if (def) {  // A-DEF1: the sweep runs on p - A Z y
      launch_def_pre_dd(c, 0, nullptr, s->pd.p, nullptr, nullptr, st);
      launch_def_in_dd(c, (int)n, s->pd.p, c.tmp_dd, nullptr, st);
      in = c.tmp_dd;
      SolverDev d3 = d0;
      d3.def_y = c.y_dd;
      fused = s->cfg.precond == PG_PREC_ILU0 &&
              launch_ilu0_apply_def_dd(d3, in, s->phd.p, nullptr, st);
    }
    if (fused)
      ;
    else if (s->cfg.precond == PG_PREC_ILU0)
      launch_ilu0_apply_dd(0, d0, nullptr, in, nullptr, s->phd.p, nullptr, st);
    else
      launch_dd_diag_apply(0, (int)n, s->cfg.precond == PG_PREC_JACOBI ? s->jdinv_dd.p : nullptr,
                           nullptr, in, nullptr, s->phd.p, nullptr, st);
    if (def && !fused)
      launch_coarse_add_dd(c, s->phd.p, nullptr, st);
    else if (!def && s->coarse_on)
      launch_coarse_apply_dd(c, s->pd.p, s->phd.p,
                             s->cfg.precond == PG_PREC_ILU0 && d.dd_stream,
                             nullptr, st);
    launch_dd_join((int)n, s->phd.p, 1.0, s->ph.p, st);
  } else {
    if (s->coarse_on && s->cfg.coarse == 2) {
      const CoarseDev c = s->coarse();
      SolverDev d0 = d;
      d0.csum = nullptr;
      launch_def_pre(c, 0, nullptr, s->p.p, nullptr, nullptr, st);
      launch_def_in(c, d.n, s->p.p, c.tmp, nullptr, st);
      SolverDev d3 = d0;
      d3.def_y = c.y;
      if (!(s->cfg.precond == PG_PREC_ILU0 &&
            launch_ilu0_apply_def(d3, c.tmp, s->ph.p, nullptr, st))) {
        launch_precond<double, double>(s->cfg.precond, 0, d0, s->jdinv.p,
                                       nullptr, c.tmp, nullptr, s->ph.p,
                                       nullptr, st);
        launch_coarse_add(c, s->ph.p, nullptr, st);
      }
    } else {
      launch_precond<double, double>(s->cfg.precond, 0, d, s->jdinv.p, nullptr,
                                     s->p.p, nullptr, s->ph.p, nullptr, st);
      if (s->coarse_on)
        launch_coarse_apply(s->coarse(), s->p.p, s->ph.p,
                            s->cfg.precond == PG_PREC_ILU0 && d.smem64 > 0,
                            nullptr, st);
    }
  }
  launch_unpermute_vec((int)n, s->perm.p, s->ph.p, s->t.p, st);
  PG_CUDA(cudaGetLastError());
  PG_CUDA(copy_out(z, s->t.p, n * sizeof(double), ptr_kind));
  PG_CUDA(cudaStreamSynchronize(st));
  int timed_out = 0;
  PG_CUDA(cudaMemcpy(&timed_out, s->err.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (timed_out) {
    PG_CUDA(cudaMemset(s->err.p, 0, sizeof(int)));
    set_error("pg_solver_apply_precond: a bounded device wait ran out");
    return PG_TIMEOUT;
  }
  return PG_OK;
}

extern "C" int pg_solver_sweep_form(const pg_solver *s) {
  if (!s || !s->analysed || s->cfg.precond != PG_PREC_ILU0) return -1;
  return s->dev().n_lgrp > 0 ? 1 : 0;
}

extern "C" int pg_solver_partition(const pg_solver *s, int32_t *part,
                                   int *n_parts) {
  PG_CHECK_ARG(s && s->analysed, "pg_solver_partition: nothing analysed");
  if (part) std::copy(s->a.part.begin(), s->a.part.end(), part);
  if (n_parts) *n_parts = s->a.n_sub;
  return PG_OK;
}

extern "C" int pg_solver_coarse_inverse(pg_solver *s, float *out, int *k) {
  PG_CHECK_ARG(s && s->analysed && s->coarse_on,
               "pg_solver_coarse_inverse: no coarse space");
  int rj = join_factor(s);
  if (!rj) rj = join_coarse(s);
  if (rj) return rj;
  const size_t K = s->a.n_sub;
  if (k) *k = (int)K;
  if (out) {
    cudaStream_t st = stream();
    PG_CUDA(cudaMemcpyAsync(out, s->ac_buf(s->ac_ready), K * K * sizeof(float),
                            cudaMemcpyDeviceToHost, st));
    PG_CUDA(cudaStreamSynchronize(st));
  }
  return PG_OK;
}

// ------------------------------------------------------------ batched solves
// Many independent systems (different sizes and patterns) stacked block-
// diagonally: one analysis (every Schwarz subdomain inside one system), one
// ILU(0) factorisation launch, and BiCGStab kernels whose CTAs each own a
// tile of one system's rows with per-system scalars (batch.cu).  The
// iteration runs as one CUDA graph launch: a WHILE conditional node
// repeats a chunk of kChunk iterations until the device-side check finds
// every system stopped (bounded by the chunk budget).  Tile shape (threads
// per CTA and rows per thread) is chosen per batch by timing the candidate
// shapes on the batch's own SpMV.
struct pg_batch {
  pg_solver *s = nullptr;  // analysis, factor and vector storage
  int n_sys = 0;
  std::vector<int64_t> sys_rows;      // original row offsets
  std::vector<uint64_t> eqn_ids;      // pattern ids of set_eqns systems
  std::vector<int32_t> h_tile_ptr;
  DevBuf<int32_t> sub_sys, tile_sys, tile_r0, tile_r1, tile_ptr;
  DevBuf<double> partials, st_vals, st_rhs;
  DevBuf<unsigned int> tickets;
  DevBuf<KScalars> sc;
  DevBuf<int> flags, chunks;  // flags: [n_sys] init / replacement selector
  KScalars *sc_host = nullptr;
  int *flags_host = nullptr;
  int block = 256, rpt = 1, n_tiles = 0;
  bool persistent = false;
  cudaGraphExec_t exec = nullptr;
  int max_chunks = 0;
  // block-diagonal coarse space (cfg.coarse): first subdomain and block
  // offset per system, coupling structure, the blocks, subdomain sums
  bool coarse = false;
  int max_k = 0;
  int64_t n_blk = 0;
  DevBuf<int32_t> c_k0, c_sub_ptr, c_cptr, c_cnb;
  DevBuf<int64_t> c_off;
  DevBuf<uint8_t> c_slot;
  DevBuf<float> c_ac;
  DevBuf<float2> c_sum;
  DevBuf<int32_t> c_azp, c_azj;
  DevBuf<uint8_t> c_azslot;
  DevBuf<double> c_azv, c_y, c_tmp;
  bool deflated() const { return coarse && s->cfg.coarse == 2; }

  ~pg_batch() {
    if (exec) cudaGraphExecDestroy(exec);
    if (sc_host) cudaFreeHost(sc_host);
    if (flags_host) cudaFreeHost(flags_host);
    if (s) pg_solver_destroy(s);
  }
  BatchTiles tiles() const {
    return BatchTiles{tile_sys.p, tile_r0.p, tile_r1.p, tile_ptr.p, n_tiles};
  }
  BatchRed red() const { return BatchRed{partials.p, tickets.p, n_tiles}; }
  SolverDev dev() const {
    SolverDev d = s->dev();
    d.sub_sys = sub_sys.p;
    d.csum = coarse ? c_sum.p : nullptr;
    return d;
  }
  CoarseBatchDev coarse_dev() const {
    CoarseBatchDev c;
    c.n_sys = n_sys;
    c.max_cnb = s->a.max_cnb;
    c.max_k = max_k;
    c.k0 = c_k0.p;
    c.off = c_off.p;
    c.sub_ptr = c_sub_ptr.p;
    c.cptr = c_cptr.p;
    c.cnb = c_cnb.p;
    c.cslot = c_slot.p;
    c.sub_sys = sub_sys.p;
    c.ac = c_ac.p;
    c.csum = c_sum.p;
    c.azp = c_azp.p;
    c.azj = c_azj.p;
    c.azv = c_azv.p;
    c.y = c_y.p;
    return c;
  }
};

namespace {

// permuted row range of every system
std::vector<int32_t> sys_prow(const pg_batch *b) {
  const Analysis &a = b->s->a;
  std::vector<int32_t> pr(b->n_sys + 1, (int32_t)a.n);
  // subdomains are grouped by system in system order
  std::vector<int32_t> first(b->n_sys, -1);
  for (int k = 0; k < a.n_sub; ++k) {
    const int32_t row = a.perm[a.sub_ptr[k]];
    const int sys = (int)(std::upper_bound(b->sys_rows.begin(),
                                           b->sys_rows.end(), (int64_t)row) -
                          b->sys_rows.begin()) - 1;
    if (first[sys] < 0) first[sys] = a.sub_ptr[k];
  }
  for (int i = b->n_sys - 1; i >= 0; --i)
    pr[i] = first[i] >= 0 ? first[i] : pr[i + 1];
  return pr;
}

int build_tiles(pg_batch *b, int block, int rpt) {
  const std::vector<int32_t> pr = sys_prow(b);
  std::vector<int32_t> ts, t0, t1, tp(b->n_sys + 1, 0);
  const int64_t tr = (int64_t)block * rpt;
  for (int i = 0; i < b->n_sys; ++i) {
    for (int64_t r = pr[i]; r < pr[i + 1]; r += tr) {
      ts.push_back(i);
      t0.push_back((int32_t)r);
      t1.push_back((int32_t)std::min<int64_t>(r + tr, pr[i + 1]));
    }
    tp[i + 1] = (int32_t)ts.size();
  }
  cudaError_t e = b->tile_sys.upload(ts);
  if (e == cudaSuccess) e = b->tile_r0.upload(t0);
  if (e == cudaSuccess) e = b->tile_r1.upload(t1);
  if (e == cudaSuccess) e = b->tile_ptr.upload(tp);
  b->n_tiles = (int)ts.size();
  if (e == cudaSuccess) e = b->partials.reserve((size_t)kMaxDots * std::max(1, b->n_tiles));
  if (e != cudaSuccess) return cuda_fail(e, "batch tiles", __FILE__, __LINE__);
  b->h_tile_ptr = tp;
  b->block = block;
  b->rpt = rpt;
  return PG_OK;
}

// Tile-shape autotuner: every candidate times the batched SpMV (the
// dominant row kernel) on this batch's matrix; the fastest shape is kept.
int autotune(pg_batch *b) {
  static const int cand[][2] = {{128, 1}, {128, 2}, {128, 4}, {256, 1},
                                {256, 2}, {256, 4}, {512, 1}, {512, 2}};
  cudaStream_t st = stream();
  pg_solver *s = b->s;
  const int64_t n = s->a.n;
  // benign scalars: running, finite
  for (int i = 0; i < b->n_sys; ++i) {
    KScalars k{};
    k.rho = k.alpha = k.omega = k.beta = k.rho_prev = 1.;
    k.max_iter = 1 << 30;
    b->sc_host[i] = k;
  }
  PG_CUDA(cudaMemcpyAsync(b->sc.p, b->sc_host, b->n_sys * sizeof(KScalars),
                          cudaMemcpyHostToDevice, st));
  // generic non-zero vectors, so no system takes a breakdown exit
  k_fill_profile<<<grid_for(n), 256, 0, st>>>(n, s->ph.p, nullptr, 1);
  k_fill_profile<<<grid_for(n), 256, 0, st>>>(n, s->rh.p, nullptr, 2);
  count_launches(2);
  float best = 1e30f;
  int bb = 256, br = 1;
  for (const auto &c : cand) {
    int rc = build_tiles(b, c[0], c[1]);
    if (rc) return rc;
    auto run = [&] {
      launch_b_spmv_v(b->tiles(), b->red(), b->block, b->dev(),
                      s->pvals.p, s->ph.p, s->v.p, s->rh.p, b->sc.p, st);
    };
    run();
    PG_CUDA(cudaEventRecord(s->ev[0], st));
    for (int k = 0; k < 5; ++k) run();
    PG_CUDA(cudaEventRecord(s->ev[1], st));
    PG_CUDA(cudaEventSynchronize(s->ev[1]));
    PG_CUDA(cudaGetLastError());
    float ms = 0.f;
    cudaEventElapsedTime(&ms, s->ev[0], s->ev[1]);
    if (ms < best) {
      best = ms;
      bb = c[0];
      br = c[1];
    }
  }
  return build_tiles(b, bb, br);
}

// Analysis of the stacked pattern (when it changed) and the per-batch
// device state.
int batch_analyse(pg_batch *b, const std::vector<int32_t> &rp,
                  const std::vector<int32_t> &ci, const double *cx,
                  const double *cy) {
  pg_solver *s = b->s;
  const int64_t n = (int64_t)rp.size() - 1;
  const int sub_rows = s->cfg.subdomain_rows ? s->cfg.subdomain_rows
                       : s->cfg.coarse           ? 512
                                                 : 1024;
  int rc = analyse(n, rp.data(), ci.data(), sub_rows, s->a, &b->sys_rows, cx,
                   cy, ilu_fill_of(s->cfg));
  if (rc) return rc;
  s->rank = n;
  rc = upload_analysis(s);
  if (rc) return rc;
  s->eqn_pattern = 0;
  // system of every subdomain
  std::vector<int32_t> ss(s->a.n_sub);
  for (int k = 0; k < s->a.n_sub; ++k) {
    const int32_t row = s->a.perm[s->a.sub_ptr[k]];
    ss[k] = (int32_t)(std::upper_bound(b->sys_rows.begin(), b->sys_rows.end(),
                                       (int64_t)row) - b->sys_rows.begin()) - 1;
  }
  PG_CUDA(b->sub_sys.upload(ss));
  b->coarse = false;
  if (s->cfg.coarse) {
    // subdomains are grouped by system in system order
    const Analysis &a = s->a;
    std::vector<int32_t> k0(b->n_sys + 1, a.n_sub);
    for (int k = a.n_sub - 1; k >= 0; --k) k0[ss[k]] = k;
    for (int t = b->n_sys - 1; t >= 0; --t)
      if (k0[t] == a.n_sub || k0[t] > k0[t + 1]) k0[t] = k0[t + 1];
    std::vector<int64_t> off(b->n_sys + 1, 0);
    b->max_k = 0;
    for (int t = 0; t < b->n_sys; ++t) {
      const int64_t kt = k0[t + 1] - k0[t];
      b->max_k = std::max<int>(b->max_k, (int)kt);
      off[t + 1] = off[t] + kt * kt;
    }
    PG_CHECK_ARG(b->max_k <= 4096,
                 "batched coarse correction: a system has more than 4096 "
                 "subdomains (raise subdomain_rows)");
    PG_CHECK_ARG(a.max_cnb <= kMaxCoarseNb,
                 "batched coarse correction: a subdomain couples to more "
                 "than 32 others");
    b->n_blk = off[b->n_sys];
    PG_CUDA(b->c_k0.upload(k0));
    PG_CUDA(b->c_off.upload(off));
    PG_CUDA(b->c_sub_ptr.upload(a.sub_ptr));
    PG_CUDA(b->c_cptr.upload(a.cptr));
    PG_CUDA(b->c_cnb.upload(a.cnb));
    PG_CUDA(b->c_slot.upload(a.cslot));
    PG_CUDA(b->c_ac.reserve((size_t)b->n_blk));
    PG_CUDA(b->c_sum.reserve((size_t)a.n_sub));
    if (s->cfg.coarse == 2) {
      PG_CUDA(b->c_azp.upload(a.azp));
      PG_CUDA(b->c_azj.upload(a.azj));
      PG_CUDA(b->c_azslot.upload(a.azslot));
      PG_CUDA(b->c_azv.reserve(a.azj.size()));
      PG_CUDA(b->c_y.reserve((size_t)a.n_sub));
      PG_CUDA(b->c_tmp.reserve((size_t)a.n));
    }
    b->coarse = true;
  }
  PG_CUDA(b->sc.reserve(b->n_sys));
  PG_CUDA(b->tickets.zero(b->n_sys));
  PG_CUDA(b->flags.reserve(b->n_sys));
  PG_CUDA(b->chunks.zero(1));
  if (b->sc_host) cudaFreeHost(b->sc_host);
  if (b->flags_host) cudaFreeHost(b->flags_host);
  b->sc_host = nullptr;
  b->flags_host = nullptr;
  PG_CUDA(cudaMallocHost((void **)&b->sc_host, b->n_sys * sizeof(KScalars)));
  PG_CUDA(cudaMallocHost((void **)&b->flags_host, b->n_sys * sizeof(int)));
  if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  return PG_OK;
}

// The whole iteration as one graph: WHILE(cond) { kChunk iterations; check }
int build_batch_graph(pg_batch *b) {
  cudaStream_t st = stream();
  pg_solver *s = b->s;
  const SolverDev d = b->dev();
  SolverDev d0 = d;  // the deflated form's sweep needs no subdomain sums
  d0.csum = nullptr;
  const CoarseBatchDev cb = b->coarse_dev();
  const BatchTiles T = b->tiles();
  const BatchRed R = b->red();
  cudaGraph_t g = nullptr;
  PG_CUDA(cudaGraphCreate(&g, 0));
  cudaGraphConditionalHandle h;
  cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
  cudaGraphNodeParams prm = {};
  prm.type = cudaGraphNodeTypeConditional;
  prm.conditional.handle = h;
  prm.conditional.type = cudaGraphCondTypeWhile;
  prm.conditional.size = 1;
  cudaGraphNode_t node;
  if (e == cudaSuccess) e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &prm);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    return cuda_fail(e, "batch graph conditional node", __FILE__, __LINE__);
  }
  cudaGraph_t body = prm.conditional.phGraph_out[0];
  const uint64_t before = launch_count();
  e = cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0,
                                    cudaStreamCaptureModeRelaxed);
  if (e == cudaSuccess) {
    for (int c = 0; c < kChunk; ++c) {
      if (b->deflated()) {
        launch_def_pre_b(cb, d.n_sub, 1, s->r.p, s->p.p, s->v.p, b->c_tmp.p,
                         b->sc.p, st);
        launch_precond<double, double>(PG_PREC_ILU0, 0, d0, nullptr, s->r.p,
                                       b->c_tmp.p, s->v.p, s->ph.p, b->sc.p, st);
        launch_coarse_add_b(cb, d.n_sub, s->ph.p, b->sc.p, st);
      } else {
        launch_precond<double, double>(PG_PREC_ILU0, 1, d, nullptr, s->r.p,
                                       s->p.p, s->v.p, s->ph.p, b->sc.p, st);
        if (b->coarse)
          launch_coarse_apply_b(cb, d.n_sub, s->p.p, s->ph.p, d.smem64 > 0,
                                b->sc.p, st);
      }
      launch_b_spmv_v(T, R, b->block, d, s->pvals.p, s->ph.p, s->v.p,
                      s->rh.p, b->sc.p, st);
      if (b->deflated()) {
        launch_def_pre_b(cb, d.n_sub, 2, s->r.p, s->s.p, s->v.p, b->c_tmp.p,
                         b->sc.p, st);
        launch_precond<double, double>(PG_PREC_ILU0, 0, d0, nullptr, s->r.p,
                                       b->c_tmp.p, s->v.p, s->sh.p, b->sc.p, st);
        launch_coarse_add_b(cb, d.n_sub, s->sh.p, b->sc.p, st);
      } else {
        launch_precond<double, double>(PG_PREC_ILU0, 2, d, nullptr, s->r.p,
                                       s->s.p, s->v.p, s->sh.p, b->sc.p, st);
        if (b->coarse)
          launch_coarse_apply_b(cb, d.n_sub, s->s.p, s->sh.p, d.smem64 > 0,
                                b->sc.p, st);
      }
      launch_b_spmv_t(T, R, b->block, d, s->pvals.p, s->sh.p, s->t.p,
                      s->s.p, b->sc.p, st);
      launch_b_update(T, R, b->block, s->x.p, s->r.p, s->ph.p, s->sh.p,
                      s->s.p, s->t.p, s->rh.p, b->sc.p, st);
    }
    launch_b_fix(T, R, b->block, s->prp.p, s->pci.p, s->pvals.p, s->b.p,
                 s->x.p, s->r.p, s->rh.p, s->p.p, s->v.p, b->sc.p, st);
    launch_b_check(b->n_sys, b->sc.p, b->chunks.p, b->max_chunks, h, st);
    cudaGraph_t captured = nullptr;
    e = cudaStreamEndCapture(st, &captured);
  }
  // capture issues nothing: the replays are counted per chunk at solve time
  count_launches(-(int)(launch_count() - before));
  if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    b->exec = nullptr;
    return cuda_fail(e, "batch graph", __FILE__, __LINE__);
  }
  b->persistent = true;
  return PG_OK;
}

}  // namespace

extern "C" int pg_batch_create(const pg_solver_cfg *cfg, pg_batch **out) {
  PG_CHECK_ARG(out, "pg_batch_create: out is NULL");
  *out = nullptr;
  pg_solver_cfg c;
  pg_solver_default_cfg(&c);
  if (cfg) c = *cfg;
  PG_CHECK_ARG(c.precond == PG_PREC_ILU0,
               "pg_batch_create: batched solves use the Schwarz ILU(0) "
               "preconditioner");
  PG_CHECK_ARG(c.precision == PG_FP64,
               "pg_batch_create: batched solves run in FP64");
  auto *b = new (std::nothrow) pg_batch();
  PG_CHECK_ARG(b, "pg_batch_create: out of host memory");
  int rc = pg_solver_create(&c, &b->s);
  if (rc) {
    delete b;
    return rc;
  }
  b->s->batch_mode = true;
  *out = b;
  return PG_OK;
}

extern "C" int pg_batch_destroy(pg_batch *b) {
  if (b) cudaStreamSynchronize(stream());
  delete b;
  return PG_OK;
}

extern "C" int pg_batch_set_eqns(pg_batch *b, int n_systems,
                                 const pg_eqn *const *eqns) {
  PG_CHECK_ARG(b && eqns && n_systems > 0, "pg_batch_set_eqns: bad argument");
  std::vector<uint64_t> ids(n_systems);
  std::vector<int64_t> rows(n_systems + 1, 0), ents(n_systems + 1, 0);
  for (int i = 0; i < n_systems; ++i) {
    PG_CHECK_ARG(eqns[i] && !eqns[i]->momentum,
                 "pg_batch_set_eqns: NULL or momentum equation");
    ids[i] = eqns[i]->pattern_id;
    rows[i + 1] = rows[i] + eqns[i]->p.n;
    ents[i + 1] = ents[i] + eqns[i]->p.nnz;
  }
  PG_CHECK_ARG(rows[n_systems] < ((int64_t)1 << 31) &&
                   ents[n_systems] < ((int64_t)1 << 31),
               "pg_batch_set_eqns: batch too large");
  pg_solver *s = b->s;
  cudaStream_t st = stream();
  if (!s->analysed || ids != b->eqn_ids) {
    b->n_sys = n_systems;
    b->sys_rows = rows;
    std::vector<int32_t> rp(rows[n_systems] + 1, 0), ci(ents[n_systems]);
    for (int i = 0; i < n_systems; ++i) {
      const EqnPattern &p = eqns[i]->p;
      for (int64_t r = 0; r < p.n; ++r)
        rp[rows[i] + r + 1] = (int32_t)(ents[i] + p.row_ptr[r + 1]);
      for (int64_t k = 0; k < p.nnz; ++k)
        ci[ents[i] + k] = (int32_t)(p.col_ind[k] + rows[i]);
    }
    // cell centres of every system (each system's subdomains are cut
    // inside its own row range)
    std::vector<double> cx(rows[n_systems]), cy(rows[n_systems]);
    bool xy = true;
    for (int i = 0; i < n_systems && xy; ++i) {
      const pg::HostMesh &hm = eqns[i]->mesh->h;
      xy = eqns[i]->p.n == hm.n_cells;
      if (xy) {
        std::copy(hm.cx.begin(), hm.cx.end(), cx.begin() + rows[i]);
        std::copy(hm.cy.begin(), hm.cy.end(), cy.begin() + rows[i]);
      }
    }
    int rc = batch_analyse(b, rp, ci, xy ? cx.data() : nullptr,
                           xy ? cy.data() : nullptr);
    if (rc) return rc;
    b->eqn_ids = ids;
    PG_CUDA(b->st_vals.reserve(ents[n_systems]));
    PG_CUDA(b->st_rhs.reserve(rows[n_systems]));
    // values for the autotuner's timing
    for (int i = 0; i < n_systems; ++i)
      PG_CUDA(cudaMemcpyAsync(b->st_vals.p + ents[i], eqns[i]->vals.p,
                              eqns[i]->p.nnz * sizeof(double),
                              cudaMemcpyDeviceToDevice, st));
    launch_permute_values((int)s->a.nnz, s->psrc.p, b->st_vals.p, s->pvals.p,
                          (int)s->a.dup_dst.size(), s->dup_dst.p,
                          s->dup_src.p, st);
    rc = autotune(b);
    if (rc) return rc;
  }
  for (int i = 0; i < n_systems; ++i) {
    PG_CUDA(cudaMemcpyAsync(b->st_vals.p + ents[i], eqns[i]->vals.p,
                            eqns[i]->p.nnz * sizeof(double),
                            cudaMemcpyDeviceToDevice, st));
    PG_CUDA(cudaMemcpyAsync(b->st_rhs.p + rows[i], eqns[i]->rhs.p,
                            eqns[i]->p.n * sizeof(double),
                            cudaMemcpyDeviceToDevice, st));
  }
  launch_permute_values((int)s->a.nnz, s->psrc.p, b->st_vals.p, s->pvals.p,
                        (int)s->a.dup_dst.size(), s->dup_dst.p, s->dup_src.p,
                        st);
  // the solver receives -rhs_ (FiniteVolumeEquation.tpp:73)
  launch_permute_vec((int)s->a.n, s->perm.p, b->st_rhs.p, -1.0, s->b.p, st);
  PG_CUDA(cudaGetLastError());
  s->have_vals = true;
  s->have_rhs = true;
  s->factored = false;
  s->eqn_src = nullptr;
  return PG_OK;
}

extern "C" int pg_batch_solve(pg_batch *b, pg_solve_stats *stats,
                              double *ms_total) {
  PG_CHECK_ARG(b && b->s && b->s->analysed && b->s->have_vals && b->s->have_rhs,
               "pg_batch_solve: set the systems first");
  pg_solver *s = b->s;
  cudaStream_t st = stream();
  const int64_t n = s->a.n;
  const int S = b->n_sys;
  const SolverDev d = b->dev();
  const BatchTiles T = b->tiles();
  const BatchRed R = b->red();
  b->max_chunks = (s->cfg.max_iters + kChunk - 1) / kChunk + 1;
  if (!b->exec) {
    int rc = build_batch_graph(b);
    if (rc) return rc;
  }
  PG_CUDA(cudaEventRecord(s->ev[0], st));
  PG_CUDA(cudaMemsetAsync(s->bad.p, 0, sizeof(int), st));
  launch_ilu0_factor(d, s->pvals.p, s->bad.p, false, st);
  if (b->coarse)
    launch_coarse_setup_b(b->coarse_dev(), d.n_sub, b->n_blk, s->pvals.p,
                          s->prp.p, st);
  if (b->deflated()) {
    CoarseDev c;
    c.azp = b->c_azp.p;
    c.azslot = b->c_azslot.p;
    c.azv = b->c_azv.p;
    launch_az_values(c, (int)n, s->prp.p, s->pvals.p, st);
  }
  for (int i = 0; i < S; ++i) {
    KScalars k{};
    k.tol2 = s->cfg.tolerance * s->cfg.tolerance;
    k.max_iter = s->cfg.max_iters;
    b->sc_host[i] = k;
    b->flags_host[i] = 1;
  }
  PG_CUDA(cudaMemcpyAsync(b->sc.p, b->sc_host, S * sizeof(KScalars),
                          cudaMemcpyHostToDevice, st));
  PG_CUDA(cudaMemcpyAsync(b->flags.p, b->flags_host, S * sizeof(int),
                          cudaMemcpyHostToDevice, st));
  PG_CUDA(cudaMemsetAsync(s->x.p, 0, n * sizeof(double), st));
  launch_b_init(T, R, b->block, s->prp.p, s->pci.p, s->pvals.p, s->b.p,
                nullptr, s->r.p, s->rh.p, s->p.p, s->v.p, b->sc.p, b->flags.p,
                st);
  for (;;) {
    PG_CUDA(cudaMemsetAsync(b->chunks.p, 0, sizeof(int), st));
    PG_CUDA(cudaGraphLaunch(b->exec, st));
    // the graph's launches are counted when it was captured; count the
    // replays by the chunks the device ran
    int ch = 0;
    PG_CUDA(cudaMemcpyAsync(&ch, b->chunks.p, sizeof(int),
                            cudaMemcpyDeviceToHost, st));
    // confirm every converged system on its true residual
    launch_b_true_residual(T, R, b->block, s->prp.p, s->pci.p, s->pvals.p,
                           s->b.p, s->x.p, nullptr, nullptr, b->sc.p, nullptr,
                           st);
    PG_CUDA(cudaMemcpyAsync(b->sc_host, b->sc.p, S * sizeof(KScalars),
                            cudaMemcpyDeviceToHost, st));
    PG_CUDA(cudaStreamSynchronize(st));
    count_launches(((b->deflated() ? 13 : b->coarse ? (d.smem64 > 0 ? 7 : 9) : 5) *
                    kChunk + 2) * ch);
    break;
  }
  launch_unpermute_vec((int)n, s->perm.p, s->x.p, s->xout.p, st);
  PG_CUDA(cudaEventRecord(s->ev[2], st));
  PG_CUDA(cudaEventSynchronize(s->ev[2]));
  PG_CUDA(cudaGetLastError());
  float ms = 0.f;
  cudaEventElapsedTime(&ms, s->ev[0], s->ev[2]);
  if (ms_total) *ms_total = ms;
  int timed_out = 0;
  PG_CUDA(cudaMemcpy(&timed_out, s->err.p, sizeof(int), cudaMemcpyDeviceToHost));
  if (timed_out) PG_CUDA(cudaMemset(s->err.p, 0, sizeof(int)));
  int worst = PG_OK;
  for (int i = 0; i < S; ++i) {
    const KScalars &k = b->sc_host[i];
    const double rel = k.bb > 0. ? std::sqrt(k.rr_true / k.bb) : 0.;
    int status = k.status;
    if (status == PG_OK && !(rel <= s->cfg.tolerance)) status = PG_MAX_ITERS;
    if (!std::isfinite(rel)) status = PG_NON_FINITE;
    if (timed_out) status = PG_TIMEOUT;
    if (stats) {
      stats[i].iters = k.iter;
      stats[i].outer_iters = k.restarts + 1;
      stats[i].status = status;
      stats[i].fp64_iters = 0;
      stats[i].rel_residual = rel;
      stats[i].ms = ms;
      stats[i].setup_ms = 0.;
    }
    if (status != PG_OK && worst == PG_OK) worst = status;
  }
  if (worst != PG_OK)
    set_error("pg_batch_solve: a system stopped with status " +
              std::to_string(worst));
  return worst;
}

extern "C" int pg_batch_get_x(const pg_batch *b, int system, double *x,
                              int ptr_kind) {
  PG_CHECK_ARG(b && x && system >= 0 && system < b->n_sys,
               "pg_batch_get_x: bad argument");
  const int64_t r0 = b->sys_rows[system], r1 = b->sys_rows[system + 1];
  PG_CUDA(copy_out(x, b->s->xout.p + r0, (r1 - r0) * sizeof(double), ptr_kind));
  PG_CUDA(cudaStreamSynchronize(stream()));
  return PG_OK;
}

extern "C" int pg_batch_tuning(const pg_batch *b, int *block,
                               int *rows_per_thread, int *n_tiles) {
  PG_CHECK_ARG(b, "pg_batch_tuning: NULL batch");
  if (block) *block = b->block;
  if (rows_per_thread) *rows_per_thread = b->rpt;
  if (n_tiles) *n_tiles = b->n_tiles;
  return PG_OK;
}
