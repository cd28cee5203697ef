// Host tree builder: box hierarchy, neighbour slots, ordered interaction
// lists with vertex flags, and the leaf-order point permutation, built to be
// identical (bit for bit, as integers) to the reference's tree.
//
// Reference behaviour reproduced here:
//  * box numbering: child c of box k is 2^d k + c (createTree,
//    1D/codes/HODLR1Dtree.hpp:79-113, 2D/codes/HODLR2Dtree.hpp:104-140,
//    3D/codes/HODLR3Dtree.hpp:116-152);
//  * child positions: 2D 0(-,-) 1(+,-) 2(+,+) 3(-,+); 3D the same at z-,
//    then 4..7 at z+ (assign_center_location, 2D :426-449, 3D :1700-1741);
//  * neighbour slots: 1D siblings only (slot 0 left, 1 right,
//    1D/codes/HODLR1Dtree.hpp:116-147); 2D edge neighbours 0 y-, 1 x+, 2 y+,
//    3 x- (2D :142-407); 3D face and edge neighbours in lexicographic 3x3x3
//    slot order, z slowest, x fastest, self removed (3D :155-1666);
//  * interaction list of a child: the children of its parent and of the
//    parent's neighbours (parent first, then neighbour slots in order) that
//    are neither the child nor its neighbours. 2D lists each group in child
//    order. The 3D tables list a group that contains some neighbour of the
//    child with its corner-sharing box first, then the others in child
//    order; groups without neighbours are in child order;
//  * vertex flag: corner-sharing entries (separate_vertex_interaction,
//    2D :452-475, 3D :1744-1767: centre distance 2*sqrt(d)*radius);
//  * charge locations: split on coordinate <= box centre, 3D testing z then
//    x then y, 2D x then y; each leaf keeps ascending original indices
//    (assignChargeLocations 1D :168-196, 2D :478-519, 3D :1769-1837), and
//    non-leaf lists are the concatenation of their children's.
#include <algorithm>
#include <cstdlib>
#include <stdexcept>

#include "h2w_internal.h"

namespace h2w {

static const int kOff2[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
static const int kOff3[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};

static inline int child_bit(int dim, int c, int a) {
    if (dim == 1) return c;
    if (dim == 2) return kOff2[c][a];
    return kOff3[c][a];
}

static inline int slot_of(int dim, const int *o) {
    if (dim == 2) {
        if (o[0] == 0 && o[1] == -1) return 0;
        if (o[0] == 1 && o[1] == 0) return 1;
        if (o[0] == 0 && o[1] == 1) return 2;
        if (o[0] == -1 && o[1] == 0) return 3;
        return -1;
    }
    int s = (o[2] + 1) * 9 + (o[1] + 1) * 3 + (o[0] + 1);
    return s > 13 ? s - 1 : s;
}

void build_tree(Tree &t) {
    const int dim = t.dim, nL = t.nL;
    if (dim < 1 || dim > 3 || nL < 1 || nL > (dim == 1 ? 30 : (dim == 2 ? 15 : 10)))
        throw std::invalid_argument("unsupported dimension / depth");
    t.nch = 1 << dim;
    t.nnb = dim == 1 ? 2 : (dim == 2 ? 4 : 26);
    const int nch = t.nch, nnb = t.nnb;
    t.nbox.assign((size_t)nL + 1, 0);
    for (int j = 0; j <= nL; ++j) t.nbox[(size_t)j] = (int64_t)1 << (dim * j);

    // integer coordinates per level
    std::vector<std::vector<int32_t>> ic((size_t)nL + 1);
    ic[0].assign((size_t)dim, 0);
    for (int j = 1; j <= nL; ++j) {
        ic[(size_t)j].resize((size_t)t.nbox[(size_t)j] * dim);
        for (int64_t k = 0; k < t.nbox[(size_t)j]; ++k) {
            int64_t p = k / nch;
            int c = (int)(k % nch);
            for (int a = 0; a < dim; ++a)
                ic[(size_t)j][(size_t)(k * dim + a)] = 2 * ic[(size_t)j - 1][(size_t)(p * dim + a)] + child_bit(dim, c, a);
        }
    }

    // neighbours and interaction lists
    t.nb.assign((size_t)nL + 1, {});
    t.ilp.assign((size_t)nL + 1, {});
    t.il.assign((size_t)nL + 1, {});
    t.ilv.assign((size_t)nL + 1, {});
    t.nb[0].assign((size_t)nnb, -1);
    t.ilp[0].assign(2, 0);
    for (int j = 1; j <= nL; ++j) {
        const int64_t nbj = t.nbox[(size_t)j];
        auto &nbv = t.nb[(size_t)j];
        auto &ilp = t.ilp[(size_t)j];
        auto &il = t.il[(size_t)j];
        auto &ilv = t.ilv[(size_t)j];
        nbv.assign((size_t)(nbj * nnb), -1);
        ilp.assign((size_t)nbj + 1, 0);
        const auto &pnb = t.nb[(size_t)j - 1];
        const auto &icj = ic[(size_t)j];
        for (int64_t k = 0; k < nbj; ++k) {
            int64_t par = k / nch;
            int c = (int)(k % nch);
            if (dim == 1) {
                if (c == 0) nbv[(size_t)(k * nnb + 1)] = (int32_t)(k + 1);
                else nbv[(size_t)(k * nnb + 0)] = (int32_t)(k - 1);
                ilp[(size_t)k + 1] = (int64_t)il.size();
                continue;
            }
            int64_t groups[27];
            int ng = 0;
            groups[ng++] = par;
            for (int s = 0; s < nnb; ++s) {
                int32_t q = pnb[(size_t)(par * nnb + s)];
                if (q != -1) groups[ng++] = q;
            }
            for (int g = 0; g < ng; ++g) {
                int64_t q = groups[g];
                int32_t vert[8], far[8];
                int nv = 0, nf = 0, nn = 0;
                for (int e = 0; e < nch; ++e) {
                    int64_t kk = q * nch + e;
                    if (kk == k) continue;
                    int o[3] = {0, 0, 0}, m = 0, nz = 0;
                    for (int a = 0; a < dim; ++a) {
                        o[a] = icj[(size_t)(kk * dim + a)] - icj[(size_t)(k * dim + a)];
                        m = std::max(m, std::abs(o[a]));
                        nz += o[a] != 0;
                    }
                    if (m >= 2) far[nf++] = (int32_t)kk;
                    else if (nz == dim) vert[nv++] = (int32_t)kk;
                    else {
                        nbv[(size_t)(k * nnb + slot_of(dim, o))] = (int32_t)kk;
                        ++nn;
                    }
                }
                int32_t ord[8];
                int no = 0;
                for (int i = 0; i < nv; ++i) ord[no++] = vert[i];
                for (int i = 0; i < nf; ++i) ord[no++] = far[i];
                if (!(dim == 3 && nn > 0)) std::sort(ord, ord + no);
                for (int i = 0; i < no; ++i) {
                    il.push_back(ord[i]);
                    bool isv = false;
                    for (int v = 0; v < nv; ++v) isv |= vert[v] == ord[i];
                    ilv.push_back((uint8_t)isv);
                }
            }
            ilp[(size_t)k + 1] = (int64_t)il.size();
        }
    }

    // box centres exactly as the reference computes them
    std::vector<std::vector<double>> cen((size_t)nL + 1);
    cen[0].assign((size_t)dim, 0.0);
    double rad = 1.0;
    for (int j = 1; j <= nL; ++j) {
        double shift = 0.5 * rad;
        cen[(size_t)j].resize((size_t)t.nbox[(size_t)j] * dim);
        for (int64_t k = 0; k < t.nbox[(size_t)j]; ++k) {
            int64_t p = k / nch;
            int c = (int)(k % nch);
            for (int a = 0; a < dim; ++a) {
                double pc = cen[(size_t)j - 1][(size_t)(p * dim + a)];
                cen[(size_t)j][(size_t)(k * dim + a)] = child_bit(dim, c, a) ? pc + shift : pc - shift;
            }
        }
        rad = 0.5 * rad;
    }

    // leaf of every point, then a stable counting sort into leaf order
    const int64_t N = t.N;
    std::vector<int64_t> leaf((size_t)N);
    for (int64_t i = 0; i < N; ++i) {
        const double *p = &t.pts[(size_t)(i * dim)];
        int64_t k = 0;
        for (int j = 0; j < nL; ++j) {
            const double *cc = &cen[(size_t)j][(size_t)(k * dim)];
            int child;
            if (dim == 1) child = p[0] <= cc[0] ? 0 : 1;
            else {
                int lo;
                if (p[0] <= cc[0]) lo = p[1] <= cc[1] ? 0 : 3;
                else lo = p[1] <= cc[1] ? 1 : 2;
                child = (dim == 3 && !(p[2] <= cc[2])) ? lo + 4 : lo;
            }
            k = k * nch + child;
        }
        leaf[(size_t)i] = k;
    }
    const int64_t nleaf = t.nbox[(size_t)nL];
    t.off.assign((size_t)nL + 1, {});
    auto &lo = t.off[(size_t)nL];
    lo.assign((size_t)nleaf + 1, 0);
    for (int64_t i = 0; i < N; ++i) ++lo[(size_t)leaf[(size_t)i] + 1];
    for (int64_t k = 0; k < nleaf; ++k) lo[(size_t)k + 1] += lo[(size_t)k];
    t.perm.assign((size_t)N, 0);
    std::vector<int64_t> fill(lo.begin(), lo.end() - 1);
    for (int64_t i = 0; i < N; ++i) t.perm[(size_t)fill[(size_t)leaf[(size_t)i]]++] = (int32_t)i;
    for (int j = nL - 1; j >= 0; --j) {
        auto &o = t.off[(size_t)j];
        const auto &oc = t.off[(size_t)j + 1];
        o.assign((size_t)t.nbox[(size_t)j] + 1, 0);
        for (int64_t k = 0; k <= t.nbox[(size_t)j]; ++k) o[(size_t)k] = oc[(size_t)(k * nch)];
    }
}

}  // namespace h2w
