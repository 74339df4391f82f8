// Internal declarations shared by the host code and the CUDA kernels of
// libphase_gb300.  Not part of the public C ABI (include/phase_gb300.h).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/phase_gb300.h"
#include "kernels.cuh"

namespace pg {

// ---------------------------------------------------------------- errors
void set_error(const std::string &msg);
int cuda_fail(cudaError_t e, const char *what, const char *file, int line);

#define PG_CUDA(call)                                                      \
  do {                                                                     \
    cudaError_t e_ = (call);                                               \
    if (e_ != cudaSuccess) return ::pg::cuda_fail(e_, #call, __FILE__, __LINE__); \
  } while (0)

#define PG_CHECK_ARG(cond, msg)                                            \
  do {                                                                     \
    if (!(cond)) {                                                         \
      ::pg::set_error(msg);                                                \
      return PG_BAD_ARG;                                                   \
    }                                                                      \
  } while (0)

cudaStream_t stream();

// Device buffer owned by the library (cudaMalloc / cudaFree).
template <class T> struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  // (re)allocate to hold at least count elements; contents undefined
  cudaError_t reserve(size_t count) {
    if (count <= n && p) return cudaSuccess;
    release();
    size_t bytes = (count ? count : 1) * sizeof(T) + 64;  // tail padding
    cudaError_t e = cudaMalloc((void **)&p, bytes);
    if (e == cudaSuccess) n = count;
    return e;
  }
  cudaError_t upload(const T *h, size_t count) {
    cudaError_t e = reserve(count);
    if (e != cudaSuccess) return e;
    if (!count) return cudaSuccess;
    return cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice,
                           stream());
  }
  cudaError_t upload(const std::vector<T> &v) { return upload(v.data(), v.size()); }
  cudaError_t zero(size_t count) {
    cudaError_t e = reserve(count);
    if (e != cudaSuccess) return e;
    return cudaMemsetAsync(p, 0, (count ? count : 1) * sizeof(T), stream());
  }
};

// Copy count elements from src (host or device per ptr_kind) to dst (device).
cudaError_t copy_in(void *dst, const void *src, size_t bytes, int ptr_kind);
cudaError_t copy_out(void *dst, const void *src, size_t bytes, int ptr_kind);

// ------------------------------------------------------------------ mesh
// Host mesh, built once per pg_mesh_create (FiniteVolumeGrid2D semantics).
struct HostMesh {
  int64_t n_cells = 0, n_faces = 0, n_interior = 0, n_boundary = 0;
  std::vector<double> cx, cy, vol;              // per cell
  std::vector<int32_t> fl, fr;                  // per face (fr = -1 boundary)
  std::vector<double> fcx, fcy, fnx, fny;       // per face centroid, normal
  // per-cell links: interior links then boundary links, each in face order
  std::vector<int64_t> link_ptr;
  std::vector<int32_t> link_face, link_cell;    // link_cell = -1 boundary
  std::vector<int32_t> n_interior_links;        // per cell
  // nodes and the cell -> node lists (ghost-cell IB stencils)
  std::vector<double> node_x, node_y;
  std::vector<int64_t> cptr, cind;
};

int build_host_mesh(const double *nodes_xy, int64_t n_nodes,
                    const int64_t *cptr, const int64_t *cind, int64_t n_cells,
                    HostMesh &m);

// Device geometry per face side, precomputed once per mesh so assembly
// reproduces the reference's arithmetic (coeff = gamma*dot(r,Sf)/|r|^2).
struct DevMesh {
  DevBuf<double> cx, cy, vol;
  DevBuf<int32_t> fl, fr;
  DevBuf<double> fcx, fcy, fnx, fny;
  DevBuf<double> fw;  // Face::distanceWeight per face (1 on boundaries)
  DevBuf<int64_t> link_ptr;
  DevBuf<int32_t> link_face;
};

// Mesh-static device data of the ghost-cell IB stencil builder (gcib.cu),
// made on the first IB build: the cell -> node and node -> cell lists (node
// cells in creation order, as Node::cells) and a uniform bucket grid over
// the nodes (bucket (bx, by) holds the nodes with floor((x - x0) / h) = bx,
// floor((y - y0) / h) = by) for nearest-node queries.
struct GcibMesh {
  DevBuf<int32_t> cptr, cind, nptr, ncell, bstart, bitems;
  DevBuf<double> node_x, node_y;
  double x0 = 0., y0 = 0., h = 1.;
  int nx = 1, ny = 1;
};

// One IB cell's image-point stencil as the device builds it: the four
// cells of the node nearest to the image point (st, creation order) with
// their coefficients, and the coefficient on the cell itself (has_self 0:
// none).  The row is the sum of these entries in this order.
struct GcibStencil {
  int32_t cell, circle, has_self, pad;
  int32_t st[4];
  double co[4];
  double self;
};

// Per-equation state of a ghost-cell IB equation: its boundary type and
// reference value, the current cell classes on the device, and the
// builder's scratch (counters: [0] IB cells, [1] error code, [2] first
// failing cell, [3] pattern-changed flag).
struct GcibState {
  int ib_bc = 0;
  double ib_ref = 0.;
  int n_circles = 0;
  DevBuf<int32_t> cls, new_cls, counters;
  DevBuf<int2> ib;
  DevBuf<GcibStencil> st;
  DevBuf<double> circles;
  int64_t n_ib = 0;
};

}  // namespace pg

struct pg_mesh {
  pg::HostMesh h;
  pg::DevMesh d;
  // ghost-cell IB builder data, made on first use (gcib.cu)
  mutable std::unique_ptr<pg::GcibMesh> gcib;
  mutable std::mutex gcib_mu;
  // link geometry per face side: dot(r, Sf_out) for the lCell and rCell
  // links, |r|^2, and the sign that turns the face normal into each side's
  // outward normal
  std::vector<double> dot_l, dot_r, msq;
  std::vector<int8_t> sgn_l, sgn_r;
};

namespace pg {

// ------------------------------------------------------------- equation
struct EqnPattern {
  int64_t n = 0, nnz = 0;
  std::vector<int32_t> row_ptr, col_ind;
  std::vector<int32_t> diag;  // position of diagonal per row (-1 if none)
  // face-coloured scatter schedule: faces permuted so each colour is a
  // contiguous range; per permuted face: original id and target slots.
  std::vector<int32_t> color_ptr;       // [n_colors+1]
  std::vector<int32_t> cface;           // original face id
  std::vector<int32_t> slot_lr, slot_rl, diag_l, diag_r;  // -1 if unused
  int n_interior_colors = 0;
};

// Ghost-cell immersed-boundary rows of the pressure equation: cell classes
// and, for every IB and solid cell, its row entries (CrsEquation order,
// zeros dropped) and rhs value.
struct GcibRows {
  std::vector<int32_t> cls;  // 0 fluid, 1 IB, 2 solid
  std::vector<std::vector<std::pair<int32_t, double>>> rows;  // per cell
  std::vector<double> rhs;                                    // per cell
};
// The device IB builder (gcib.cu): classify the cells of m for the circles
// (cx, cy, r per circle, host), build the stencils of the IB cells into
// st, and return the rows of the equation in g.  With check_pattern, the
// classes are compared with st.cls, and when they match the new IB rows
// are written into base_vals (the equation's pattern row_ptr/col_ind);
// *changed says whether the pattern must be rebuilt (g is filled then).
int gcib_build(const pg_mesh *m, GcibState &st, int n_circles, const double *circles,
               GcibRows &g, bool check_pattern = false,
               const int32_t *row_ptr = nullptr, const int32_t *col_ind = nullptr,
               double *base_vals = nullptr, double *base_rhs = nullptr,
               bool *changed = nullptr);

// row_mask (optional): rows with mask 0 get no Laplacian entries; extra
// (optional): entries appended to each row (the GCIB rows)
int build_pattern(const HostMesh &m, int gamma_kind, const int32_t *bc_type,
                  EqnPattern &p, bool diag_first = false,
                  const GcibRows *extra = nullptr);

}  // namespace pg

struct pg_eqn {
  const pg_mesh *mesh = nullptr;
  int gamma_kind = 0;
  pg::EqnPattern p;
  std::vector<int32_t> bc_type;
  pg::DevBuf<int32_t> row_ptr, col_ind;
  pg::DevBuf<double> vals, rhs;
  // colour-ordered face schedule on device
  pg::DevBuf<int32_t> cface, cl, cr, slot_lr, slot_rl, diag_l, diag_r;
  pg::DevBuf<int32_t> cbc;  // bc type per colour-ordered face
  pg::DevBuf<double> cdot_l, cdot_r, cmsq, csfl_x, csfl_y, csfr_x, csfr_y;
  pg::DevBuf<double> stage_a, stage_b, stage_c;  // host-input staging
  uint64_t version = 0;  // bumps on every assembly
  uint64_t pattern_id = 0;
  bool momentum = false;   // vector momentum operator: rhs holds 2n values
  bool any_fixed = false;  // a boundary face has a FIXED condition
  pg::DevBuf<int32_t> diag;  // diagonal position per row
  // ghost-cell IB equation: constant IB/solid rows the assembly starts from
  bool has_base = false;
  pg::DevBuf<double> base_vals, base_rhs;
  std::vector<int32_t> cell_class;
  std::unique_ptr<pg::GcibState> ib;  // ghost-cell IB equations only
};

namespace pg {

// --------------------------------------------------------------- analysis
// Sparsity analysis of a solver matrix: additive-Schwarz partition, level
// schedule within each subdomain and the permutation that makes every
// subdomain contiguous and level-ordered.
struct Analysis {
  int64_t n = 0;
  int64_t nnz = 0;        // entries after dropping placeholders/merging
  int64_t n_src = 0;      // length of the caller's col_ind array
  int n_sub = 0;
  int max_sub_rows = 0, max_sub_lu = 0, max_levels = 0;
  std::vector<int32_t> perm, iperm;        // new->old, old->new
  std::vector<int32_t> prp, pci, psrc;     // permuted CSR; psrc -> caller idx
  // sliced ELLPACK (32-row slices) of the permuted pattern: slice offsets,
  // columns, permuted-CSR source of each entry (-1 padding)
  std::vector<int32_t> sell_ptr, sell_col, sell_src;
  std::vector<int32_t> dup_dst, dup_src;   // extra summed duplicates
  std::vector<int32_t> sub_ptr;            // [n_sub+1] permuted row starts
  std::vector<int32_t> sub_lvl;            // [n_sub+1] index into lvl_ptr
  std::vector<int32_t> lvl_ptr;            // level row boundaries
  // ILU(0) storage restricted to subdomains
  std::vector<int32_t> lrp, ldg, lsrc;     // row ptr, diag pos, -> perm entry
  std::vector<int32_t> lci;                // subdomain-local column
  std::vector<int32_t> part;               // subdomain of each original row
  bool global_ilu = false;                 // one subdomain holding all rows
  // packed ILU(0) records (static parts filled; values by the factor)
  std::vector<SubMeta> meta64;
  std::vector<uint8_t> rec64;
  std::vector<int32_t> rec_src;            // value slot -> permuted entry
  size_t smem64 = 0;                       // max record + vector bytes
  int max_kl = 0, max_ku = 0;              // widest L / U part of a row
  // streaming records for the apply kernel (kernels.cuh StreamMeta), one
  // per sweep group
  std::vector<StreamMeta> smeta64;
  int n_grp = 0;
  std::vector<uint8_t> srec64;
  std::vector<int32_t> pack_src, pack_dst64;    // FP64 stream <- factor
  size_t ssmem64 = 0;
  // line form of the sweep records (kernels.cuh LineMeta) when every
  // subdomain is a structured block (empty otherwise)
  std::vector<LineMeta> lmeta;
  std::vector<uint8_t> lrec;
  std::vector<int32_t> lpack_src, lpack_dst;  // line record <- factor
  size_t lsmem = 0;
  // the same with FP32 weights (mixed solver, mixed_sweep 3): one forward
  // and one backward piece per group
  std::vector<LineMeta> lmeta32;
  std::vector<uint8_t> lrec32;
  std::vector<int32_t> lpack32_src, lpack32_dst;  // in 4-byte units
  size_t lsmem32 = 0;
  // float-float step stream (kernels.cuh StepMeta) of the mixed solver,
  // when every row has at most 3 L and 3 U entries
  bool use_steps = false;
  std::vector<StepMeta> tmeta_dd;
  std::vector<uint8_t> srec_dd;
  std::vector<int32_t> pack_src_dd, pack_dst_dd;  // step values <- factor
  size_t ssmem_dd = 0;
  // coarse space of the two-level Schwarz preconditioner (one indicator
  // vector per subdomain): the coarse matrix row of subdomain s has the
  // columns cnb[cptr[s] .. cptr[s+1]) (the subdomains its rows couple to,
  // ascending), and cslot[k] is the position of permuted entry k's column
  // subdomain in its row's list
  std::vector<int32_t> cptr, cnb;
  std::vector<uint8_t> cslot;
  int max_cnb = 0;
  // A Z (Z the subdomain indicators) per permuted row: the subdomains
  // azj[azp[i] .. azp[i+1]) its columns fall in, and each entry's position
  // among them (azslot[k])
  std::vector<int32_t> azp, azj;
  std::vector<uint8_t> azslot;
};

// most subdomains one coarse matrix row may couple to
constexpr int kMaxCoarseNb = 32;

// target bytes of one streamed piece of a subdomain's factor
constexpr int64_t kStreamPiece = 6144;

// sys_rows (optional): row offsets of independent systems stacked block-
// diagonally (batched solves); every subdomain then lies in one system.
// cx/cy (optional): a point per row (the cell centres of a finite-volume
// equation); ranges are then cut by coordinate bisection across their
// longer extent instead of by graph distance, which gives compact
// subdomains with short level schedules (a 32 x 32 block of a structured
// grid has 63 levels).
// fill: level of fill k of the ILU(k) blocks (0: ILU(0)).
int analyse(int64_t n, const int32_t *row_ptr, const int32_t *col_ind,
            int subdomain_rows, Analysis &a,
            const std::vector<int64_t> *sys_rows = nullptr,
            const double *cx = nullptr, const double *cy = nullptr,
            int fill = 0);

}  // namespace pg
