// Internal host-side structures of the GB300 H2* / (H2+H)* library.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/h2w.h"

namespace h2w {

// ---------------------------------------------------------------- tree ---
// Uniform 2^d-ary tree over [-1,1]^d with the reference's box numbering,
// neighbour slots and ordered interaction lists. Points are permuted into
// leaf order: box k at level j owns leaf-order positions [off[j][k], off[j][k+1]).
struct Tree {
    int dim = 0, nL = 0, nch = 0, nnb = 0;
    int64_t N = 0;
    std::vector<double> pts;                    // N*dim, original order
    std::vector<int32_t> perm;                  // leaf-order position -> original index
    std::vector<int64_t> nbox;                  // boxes per level
    std::vector<std::vector<int64_t>> off;      // per level: nbox+1 leaf-order offsets
    std::vector<std::vector<int32_t>> nb;       // per level: nbox*nnb neighbour slots (-1 = none)
    std::vector<std::vector<int64_t>> ilp;      // per level: interaction-list CSR ptr
    std::vector<std::vector<int32_t>> il;       // interaction-list boxes
    std::vector<std::vector<uint8_t>> ilv;      // 1 = vertex-sharing entry
    int64_t cnt(int j, int64_t k) const { return off[j][k + 1] - off[j][k]; }
};

void build_tree(Tree &t);

// ------------------------------------------------------------ skeleton ---
// Pivot sets per box (global point ids, pivot order) for one basis kind.
struct Skel {
    std::vector<int64_t> ptr;   // nbox+1
    std::vector<int32_t> chk;   // row pivots (check points)
    std::vector<int32_t> chg;   // column pivots (charge points)
    int64_t rank(int64_t k) const { return ptr[k + 1] - ptr[k]; }
};

// Semi-nested / 1D pair list at one level.
struct Pairs {
    std::vector<int32_t> box, slot, other;      // target box, IL slot (or sibling slot), source box
    std::vector<int64_t> ptr;                   // npairs+1
    std::vector<int32_t> row, col;              // pivots, global ids
};

// -------------------------------------------------------------- plans ---
// One block-row GEMV target: rows [dst, dst+nrows) of the workspace (or of
// the output vector through perm when flagged), computed as the sum over
// panels p of A_p (nrows x w_p, row-major, leading dimension lda_p) times
// the gathered source x_p (concatenation of the panel's segments).
enum : int32_t { T_OVERWRITE = 0, T_ACCUM = 1, T_ATOMIC = 2, T_SCATTER = 4 };
enum : int32_t { S_WS = 0, S_GATHER = 1 };

struct Target {
    int64_t dst;
    int32_t nrows, flags, p0, p1, gsz, xw;  // panels [p0,p1), lanes per row, gathered width
    int32_t ldsum, pad;                      // sum of the panels' leading dimensions
};
struct Panel {
    int64_t a;
    int32_t lda, w, s0, s1, xoff, pad;
};
struct Seg {
    int64_t src;
    int32_t len, xoff, flags, pad;
};

struct Phase {
    int64_t t0, t1;   // target range
    int max_xw;       // shared-memory words needed
    int logical = 0;  // the pass it belongs to (0 .. 2L; empty passes have no Phase)
};

// Assembly jobs.
struct FillJob {        // op[a + i*lda + c] = K(rows[i], cols[c])
    int64_t a, ri, ci;  // offsets into the index buffer
    int32_t nr, nc, lda, pad;
};
struct FactorJob {      // LU of K(I,J) (r x r) into factor buffer at f
    int64_t f, ii, jj;
    int32_t r, pad;
};
enum : int32_t { X_ROW_RL = 0, X_ROW_R = 1, X_COL_LR = 2, X_COL_L = 3 };
struct XferJob {        // rows or columns of K(.,J) solved against the LU factors at f
    int64_t f, jj, pi;  // factor, pivot list (length r), points list (length n)
    int64_t a1, a2;     // a1: row-major n x r (ld1) [ROW] or r x n (ld1) [COL]; a2: transposed copy (ld2) or -1
    int32_t r, n, ld1, ld2, mode, pad;
};

}  // namespace h2w
