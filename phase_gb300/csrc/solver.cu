// The SparseMatrixSolver replacement: sparsity analysis caching, value
// permutation, ILU(0) factorisation and the device-resident BiCGStab loop
// with reliable residual updates.  FP64 vectors and SpMV throughout; in
// PG_MIXED the ILU(0) factors are stored and swept in FP32.
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
  DevBuf<SubMeta> meta64, meta32;
  DevBuf<uint8_t> rec64, rec32;
  DevBuf<StreamMeta> smeta64, smeta32;
  DevBuf<StepMeta> tmeta32;
  DevBuf<uint8_t> srec64, srec32;
  DevBuf<int32_t> pack_src, pack_dst64, pack_src32, pack_dst32;
  DevBuf<int> err;
  DevBuf<int32_t> raw_rp, raw_ci, st_rp, st_ci;
  DevBuf<double> st_vals, st_vec;
  DevBuf<unsigned int> diff;
  // values and factors
  DevBuf<double> pvals, jdinv;
  // Krylov vectors (permuted order)
  DevBuf<double> b, x, r, rh, p, v, ph, s, sh, t, xout;
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
  // CUDA graphs of one chunk of BiCGStab iterations (FP64 and FP32 ILU
  // sweeps); kernel
  // arguments are fixed device pointers, so a graph stays valid until the
  // buffers are reallocated by a new analysis
  cudaGraphExec_t chunk_graph[2] = {nullptr, nullptr};

  void drop_graphs() {
    for (auto &g : chunk_graph)
      if (g) {
        cudaGraphExecDestroy(g);
        g = nullptr;
      }
  }

  ~pg_solver() {
    drop_graphs();
    if (sc_host) cudaFreeHost(sc_host);
    if (bad_host) cudaFreeHost(bad_host);
    if (diff_host) cudaFreeHost(diff_host);
    for (auto &e : ev)
      if (e) cudaEventDestroy(e);
  }

  SolverDev dev() const {
    SolverDev d;
    d.n = (int)a.n;
    d.nnz = (int)a.nnz;
    d.n_sub = a.n_sub;
    d.prp = prp.p;
    d.pci = pci.p;
    d.meta64 = meta64.p;
    d.meta32 = meta32.p;
    d.rec64 = rec64.p;
    d.rec32 = rec32.p;
    d.rec_src = rec_src.p;
    // the streamed (TMA) apply needs header + 2 pieces + the subdomain's
    // vector in shared memory; otherwise the global-memory sweep is used
    d.smem64 = a.ssmem64 <= kMaxApplySmem ? a.ssmem64 : 0;
    d.smem32 = a.ssmem32 <= kMaxApplySmem ? a.ssmem32 : 0;
    d.smeta64 = smeta64.p;
    d.smeta32 = smeta32.p;
    d.srec64 = srec64.p;
    d.srec32 = srec32.p;
    d.pack_src = pack_src.p;
    d.pack_dst64 = pack_dst64.p;
    d.pack_src32 = pack_src32.p;
    d.pack_dst32 = pack_dst32.p;
    d.n_pack = (int)a.pack_src.size();
    d.n_pack32 = (int)a.pack_src32.size();
    d.use_steps = a.use_steps ? 1 : 0;
    d.tmeta32 = tmeta32.p;
    d.max_kl = a.max_kl;
    d.max_ku = a.max_ku;
    d.err = err.p;
    return d;
  }
  RedWork red() const { return RedWork{partials.p, ticket.p, red_grid}; }
};

namespace {

int upload_analysis(pg_solver *s) {
  const Analysis &a = s->a;
  cudaError_t e = cudaSuccess;
  auto up = [&](auto &buf, const auto &vec) {
    if (e == cudaSuccess) e = buf.upload(vec);
  };
  up(s->perm, a.perm);
  up(s->prp, a.prp);
  up(s->pci, a.pci);
  up(s->psrc, a.psrc);
  up(s->dup_dst, a.dup_dst);
  up(s->dup_src, a.dup_src);
  up(s->rec_src, a.rec_src);
  up(s->meta64, a.meta64);
  up(s->meta32, a.meta32);
  up(s->rec64, a.rec64);
  up(s->rec32, a.rec32);
  up(s->smeta64, a.smeta64);
  up(s->tmeta32, a.tmeta32);
  up(s->smeta32, a.smeta32);
  up(s->srec64, a.srec64);
  up(s->srec32, a.srec32);
  up(s->pack_src, a.pack_src);
  up(s->pack_dst64, a.pack_dst64);
  up(s->pack_src32, a.pack_src32);
  up(s->pack_dst32, a.pack_dst32);
  if (e == cudaSuccess) e = s->err.zero(1);
  const size_t n = a.n, nnz = a.nnz;
  for (DevBuf<double> *bf : {&s->b, &s->x, &s->r, &s->rh, &s->p, &s->v,
                             &s->ph, &s->s, &s->sh, &s->t, &s->xout,
                             &s->jdinv})
    if (e == cudaSuccess) e = bf->reserve(n);
  if (e == cudaSuccess) e = s->pvals.reserve(nnz);
  s->drop_graphs();
  s->red_grid = (int)std::min<int64_t>(1216, (n + kVecBlock - 1) / kVecBlock);
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
  return PG_OK;
}

int ensure_host_state(pg_solver *s) {
  if (!s->sc_host) PG_CUDA(cudaMallocHost((void **)&s->sc_host, sizeof(KScalars)));
  if (!s->bad_host) PG_CUDA(cudaMallocHost((void **)&s->bad_host, sizeof(int)));
  if (!s->diff_host) PG_CUDA(cudaMallocHost((void **)&s->diff_host, sizeof(unsigned)));
  for (auto &e : s->ev)
    if (!e) PG_CUDA(cudaEventCreate(&e));
  return PG_OK;
}

// PG_SOLVER_TRACE=1 prints the Krylov scalars at every chunk boundary
bool trace_enabled() {
  static const int on = [] {
    const char *e = std::getenv("PG_SOLVER_TRACE");
    return e && e[0] == '1' ? 1 : 0;
  }();
  return on != 0;
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
                 int *updates) {
  cudaStream_t st = stream();
  const SolverDev d = s->dev();
  const RedWork w = s->red();
  const bool fp32_ilu =
      s->cfg.precision == PG_MIXED && s->cfg.precond == PG_PREC_ILU0;
  double *const val = s->pvals.p, *const jd = s->jdinv.p;
  double *const x = s->x.p, *const r = s->r.p, *const rh = s->rh.p;
  double *const p = s->p.p, *const v = s->v.p, *const ph = s->ph.p;
  double *const ss = s->s.p, *const sh = s->sh.p, *const t = s->t.p;
  auto precond = [&](int mode, double *pv, double *z) {
    if (fp32_ilu)
      launch_ilu0_apply_fp32(mode, d, r, pv, v, z, s->sc.p, st);
    else
      launch_precond<double, double>(s->cfg.precond, mode, d, jd, r, pv, v, z,
                                     s->sc.p, st);
  };
  // one chunk = kChunk iterations, 5 kernels each; captured once into a CUDA
  // graph after the first direct chunk and replayed
  constexpr int kChunk = 8;
  constexpr double kDelta2 = 1e-4;   // replace when rr < kDelta2 * rr_ref
  constexpr int kMaxRestarts = 50;
  auto chunk = [&]() {
    for (int c = 0; c < kChunk; ++c) {
      precond(1, p, ph);
      launch_spmv_v<double, double>(d, val, ph, v, rh, s->sc.p, w, st);
      precond(2, ss, sh);
      launch_spmv_t<double, double>(d, val, sh, t, ss, s->sc.p, w, st);
      launch_update<double>(d.n, x, r, ph, sh, ss, t, rh, s->sc.p, w, st);
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
  cudaGraphExec_t &gexec = s->chunk_graph[fp32_ilu ? 1 : 0];
  bool direct_done = false;
  for (;;) {
    if (gexec) {
      PG_CUDA(cudaGraphLaunch(gexec, st));
      count_launches(5 * kChunk);
    } else if (direct_done) {
      cudaGraph_t graph = nullptr;
      PG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
      chunk();  // launches are counted here, executed once below
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

int factor(pg_solver *s) {
  cudaStream_t st = stream();
  const SolverDev d = s->dev();
  const bool mixed = s->cfg.precision == PG_MIXED;
  if (s->cfg.precond == PG_PREC_ILU0) {
    PG_CUDA(cudaMemsetAsync(s->bad.p, 0, sizeof(int), st));
    launch_ilu0_factor(d, s->pvals.p, s->bad.p, mixed, st);
    PG_CUDA(cudaGetLastError());
  } else if (s->cfg.precond == PG_PREC_JACOBI) {
    launch_jacobi_diag(d, s->pvals.p, s->jdinv.p, st);
  }
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
    int rc = analyse(n, hrp, hci, s->cfg.precond == PG_PREC_ILU0 ? s->cfg.subdomain_rows : -1, s->a);
    if (rc) return rc;
    rc = upload_analysis(s);
    if (rc) return rc;
    PG_CUDA(s->raw_rp.upload(hrp, n + 1));
    PG_CUDA(s->raw_ci.upload(hci, n_src));
    s->eqn_pattern = 0;
  }
  launch_permute_values((int)s->a.nnz, s->psrc.p, dv, s->pvals.p,
                        (int)s->a.dup_dst.size(), s->dup_dst.p, s->dup_src.p, st);
  PG_CUDA(cudaGetLastError());
  s->have_vals = true;
  return PG_OK;
}

extern "C" int pg_solver_set_eqn(pg_solver *s, const pg_eqn *e) {
  PG_CHECK_ARG(s && e, "pg_solver_set_eqn: NULL arg");
  PG_CHECK_ARG(!e->momentum,
               "pg_solver_set_eqn: a momentum equation has two right-hand "
               "sides; use pg_solver_set_csr/set_rhs per component");
  cudaStream_t st = stream();
  if (s->rank != e->p.n) {
    s->rank = e->p.n;
    s->analysed = false;
  }
  if (!s->analysed || s->eqn_pattern != e->pattern_id) {
    int rc = analyse(e->p.n, e->p.row_ptr.data(), e->p.col_ind.data(),
                     s->cfg.precond == PG_PREC_ILU0 ? s->cfg.subdomain_rows : -1, s->a);
    if (rc) return rc;
    rc = upload_analysis(s);
    if (rc) return rc;
    s->eqn_pattern = e->pattern_id;
  }
  launch_permute_values((int)s->a.nnz, s->psrc.p, e->vals.p, s->pvals.p,
                        (int)s->a.dup_dst.size(), s->dup_dst.p, s->dup_src.p, st);
  // the solver receives -rhs_ (FiniteVolumeEquation.tpp:179)
  launch_permute_vec((int)s->a.n, s->perm.p, e->rhs.p, -1.0, s->b.p, st);
  PG_CUDA(cudaGetLastError());
  s->have_vals = true;
  s->have_rhs = true;
  return PG_OK;
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
  if (!s->have_x) PG_CUDA(cudaMemsetAsync(s->x.p, 0, n * sizeof(double), st));
  PG_CUDA(cudaEventRecord(s->ev[0], st));
  int rc = factor(s);
  if (rc) return rc;
  PG_CUDA(cudaEventRecord(s->ev[1], st));
  if (s->cfg.precond == PG_PREC_ILU0) {
    PG_CUDA(cudaMemcpyAsync(s->bad_host, s->bad.p, sizeof(int),
                            cudaMemcpyDeviceToHost, st));
  }
  int iters = 0, outer = 0;
  const double tol = s->cfg.tolerance;
  const SolverDev d = s->dev();
  const RedWork w = s->red();
  int status = run_bicgstab(s, tol, s->cfg.max_iters, &iters, &outer);
  if (status == PG_CUDA_ERROR) return status;
  const double bb = s->sc_host->bb;
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

extern "C" int pg_solver_profile(pg_solver *s, int reps, double *ms) {
  PG_CHECK_ARG(s && ms && reps > 0, "pg_solver_profile: bad argument");
  PG_CHECK_ARG(s->analysed && s->have_vals && s->have_x,
               "pg_solver_profile: solve a system first");
  cudaStream_t st = stream();
  const SolverDev d = s->dev();
  const RedWork w = s->red();
  const int64_t n = s->a.n;
  const int g = grid_for(n);
  const bool fp32_ilu =
      s->cfg.precision == PG_MIXED && s->cfg.precond == PG_PREC_ILU0;
  // scratch vectors with benign non-zero contents, so no kernel takes its
  // breakdown/convergence exit; the solver's own state is left untouched
  DevBuf<double> d8[8];
  for (int k = 0; k < 8; ++k) {
    PG_CUDA(d8[k].reserve(n));
    k_fill_profile<<<g, 256, 0, st>>>(n, d8[k].p, nullptr, k);
  }
  KScalars k{};
  k.max_iter = 1 << 30;
  k.alpha = k.omega = k.beta = k.rho = k.rho_prev = 1.0;
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
  for (int i = 0; i < 8; ++i) ms[i] = 0.;
  // vectors: 0 ph/sh, 1 v/t, 2 rh, 3 r, 4 p/s, 5 x, 6 z
  int rc = timed([&] { launch_spmv_v<double, double>(d, s->pvals.p, d8[0].p, d8[1].p, d8[2].p, s->sc.p, w, st); }, &ms[0]);
  if (!rc) rc = timed([&] { launch_precond<double, double>(s->cfg.precond, 1, d, s->jdinv.p, d8[3].p, d8[4].p, d8[1].p, d8[6].p, s->sc.p, st); }, &ms[1]);
  if (!rc) rc = timed([&] { launch_update<double>(d.n, d8[5].p, d8[3].p, d8[0].p, d8[6].p, d8[4].p, d8[1].p, d8[2].p, s->sc.p, w, st); }, &ms[2]);
  if (!rc && s->cfg.precond == PG_PREC_ILU0)
    rc = timed([&] { launch_ilu0_factor(d, s->pvals.p, s->bad.p, fp32_ilu, st); }, &ms[3]);
  if (!rc && fp32_ilu)
    rc = timed([&] { launch_ilu0_apply_fp32(1, d, d8[3].p, d8[4].p, d8[1].p, d8[6].p, s->sc.p, st); }, &ms[4]);
  PG_CUDA(cudaStreamSynchronize(st));
  return rc;
}

extern "C" int pg_solver_apply_precond(pg_solver *s, const double *r,
                                       double *z, int ptr_kind) {
  PG_CHECK_ARG(s && r && z, "pg_solver_apply_precond: NULL arg");
  PG_CHECK_ARG(s->analysed && s->have_vals,
               "pg_solver_apply_precond: set the matrix first");
  cudaStream_t st = stream();
  const SolverDev d = s->dev();
  const int64_t n = s->a.n;
  int rc = factor(s);
  if (rc) return rc;
  const double *dr = r;
  if (ptr_kind != PG_DEVICE) {
    PG_CUDA(s->st_vec.upload(r, n));
    dr = s->st_vec.p;
  }
  // z = M^-1 r in the permuted order (mode 0 reads p, writes ph)
  launch_permute_vec((int)n, s->perm.p, dr, 1.0, s->p.p, st);
  if (s->cfg.precision == PG_MIXED && s->cfg.precond == PG_PREC_ILU0)
    launch_ilu0_apply_fp32(0, d, nullptr, s->p.p, nullptr, s->ph.p, nullptr, st);
  else
    launch_precond<double, double>(s->cfg.precond, 0, d, s->jdinv.p, nullptr,
                                   s->p.p, nullptr, s->ph.p, nullptr, st);
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

extern "C" int pg_solver_partition(const pg_solver *s, int32_t *part,
                                   int *n_parts) {
  PG_CHECK_ARG(s && s->analysed, "pg_solver_partition: nothing analysed");
  if (part) std::copy(s->a.part.begin(), s->a.part.end(), part);
  if (n_parts) *n_parts = s->a.n_sub;
  return PG_OK;
}
