// Multifrontal sparse LU (the direct-solver backend): symbolic structures
// shared by the host analysis (lu_host.cpp) and the device factorisation and
// solves (lu.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

namespace pg {

// Fronts whose order is at most kLuSmallM (FP64) are assembled and
// factorised whole in shared memory by one CTA; larger ones are assembled
// in global memory and factorised in 32-column panels by batched kernels.
constexpr int kLuSmallM = 112;
// panel width of the large fronts (16 measured no faster on the 1M bubble:
// 153.6 vs 151.1 ms factorisation, and slower blocked solves)
constexpr int kLuPanel = 32;
constexpr int kLuTrsmCols = 128;  // columns of U12 per TRSM tile
constexpr int kLuUpd = 64;        // edge of a trailing-update tile

// One front (a node of the nested-dissection tree) as the kernels see it.
// Its index list is S (the k fully summed variables, new numbers s0 ..
// s0+k-1) followed by U (the m-k update variables, ascending new numbers,
// all eliminated later).  The m x m front is stored row-major at `off` in
// the factor pool; after the partial factorisation its leading k rows hold
// U11 | U12, its leading k columns below the diagonal L11 / L21 (unit
// diagonal implied), and its trailing (m-k) x (m-k) block the contribution
// block that the parent assembles.
struct LuFront {
  int32_t m, k, s0, idx;  // order, pivots, first new index, offset in fidx
  int32_t child_ptr, n_child, parent, large;
  int64_t off;   // front offset in the factor pool (elements)
  int64_t coff;  // contribution vector offset in the solve pool (m-k long)
  int32_t rel_off;   // this front's U -> parent-position map (u entries)
  int32_t inv_off;   // parent-position -> this front's U index map
                     // (parent m entries, -1 where absent); large parents
  int32_t ent_ptr, ent_end;  // range of its original entries
  int32_t first;             // smallest new index in its subtree
  int32_t pad_;
};

struct LuSymbolic {
  int64_t n = 0;
  int64_t n_src = 0;             // length of the caller's col_ind
  std::vector<int32_t> perm;     // new -> old
  std::vector<int32_t> iperm;    // old -> new
  std::vector<LuFront> fronts;   // postorder (children before parents)
  std::vector<int32_t> children; // child ids, by parent child_ptr
  std::vector<int32_t> fidx;     // index lists (new numbers)
  std::vector<int32_t> rel;      // per child: U -> position in parent front
  std::vector<int32_t> inv;      // per child of a large parent: inverse map
  // original entries: local position in the owning front (row * m + col),
  // summed over the caller indices e_src[e_ptr[e] .. e_ptr[e+1])
  std::vector<int32_t> e_pos, e_ptr, e_src;
  // column of each caller index in new numbering (-1 for placeholders):
  // used for the column scales of the pivot test
  std::vector<int32_t> src_col;
  // fronts grouped by height (leaves 0): small fronts, large fronts, and
  // the row tasks of the large fronts' assembly
  int n_heights = 0;
  std::vector<int32_t> h_small_ptr, h_small;  // [n_heights+1], front ids
  std::vector<int32_t> h_large_ptr, h_large;
  std::vector<int32_t> h_all_ptr, h_all;      // every front, by height
  std::vector<int32_t> h_maxm;                // largest order per height
  // panel tasks of large fronts: for height h and panel q the fronts with
  // k > 32 q (diag), their TRSM tiles and their update tiles
  struct PanelStep {
    int height, panel;
    int diag_ptr, diag_end;    // into pt_diag (front ids): panel CTAs
    int trsm_ptr, trsm_end;    // into pt_trsm (front, 1, first column)
    int upd_ptr, upd_end;      // into pt_upd (front, tile_i, tile_j)
  };
  std::vector<PanelStep> steps;
  std::vector<int32_t> pt_diag;
  std::vector<int32_t> pt_trsm;  // triples
  std::vector<int32_t> pt_upd;   // triples
  std::vector<int32_t> large_rows;  // (front, row) pairs for assembly
  std::vector<int32_t> h_rows_ptr;  // per height into large_rows / 2
  int64_t pool = 0;       // factor pool elements
  int64_t cpool = 0;      // contribution pool elements
  int max_m = 0, max_k = 0;
  double flops = 0.;      // factorisation flops (multiply-add = 2)
  int64_t factor_nnz = 0; // entries of L and U (fronts' k rows and columns)
};

// Nested-dissection analysis of the pattern (placeholders skipped,
// repeated columns summed).  xy (optional, 2 per row): cut by coordinate
// bisection across the longer extent; otherwise by breadth-first graph
// bisection.  leaf: largest set cut no further.
int lu_analyse(int64_t n, const int32_t *row_ptr, const int32_t *col_ind,
               const double *x, const double *y, int leaf, LuSymbolic &s);

}  // namespace pg

// The LU as an inverse builder for small dense inverses of sparse matrices
// (the two-level preconditioner's coarse matrix): analysis and buffers once
// per pattern, then per set of values a factorisation and the dense inverse
// issued on the caller's stream with no host synchronisation.
struct pg_lu;
namespace pg {
// *out = nullptr (and PG_OK) when a front is larger than kLuSmallM: the
// caller keeps its own method for such patterns
int lu_inverse_setup(int64_t n, const int32_t *row_ptr, const int32_t *col_ind,
                     pg_lu **out);
// A^-1 (row-major n x n, FP32, the caller's numbering) of the values vals
// (indexed like col_ind); FP64 factorisation, FP32 multi-right-hand-side
// triangular solves
int lu_inverse_run(pg_lu *lu, const double *vals, float *out, cudaStream_t st);
// kernels one lu_inverse_run launches; whether a captured graph of it has
// run once (launch accounting of graph replays)
int lu_inverse_launches(const pg_lu *lu);
bool lu_inverse_captured(const pg_lu *lu);
void lu_inverse_set_captured(pg_lu *lu);
}  // namespace pg
