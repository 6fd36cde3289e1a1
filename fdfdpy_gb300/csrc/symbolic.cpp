// Symbolic analysis: geometric nested dissection of the periodic Nx x Ny
// grid.  The graph is the one of construct_A's 5-point operator
// (fdfdpy/linalg.py:52-66, 69-93): cell k = i*Ny + j couples to
// (i+-1 mod Nx, j) and (i, j+-1 mod Ny) because createDws builds periodic
// differences (fdfdpy/derivatives.py:22-32, wrap diagonals at -N+1, N-1).
//
// Tree shape
//   * root front: the "cross" row 0 + column 0.  Removing it cuts every
//     wrap-around edge, leaving the open rectangle R = [1,Nx) x [1,Ny).
//   * R is bisected recursively across its longer side; each internal
//     front's pivots are one separator line, its boundary is the ring of
//     cells just outside its rectangle (all of which lie on ancestor
//     separators).  Rectangles of at most leaf_area cells become leaves
//     whose pivots are all their cells.
// Fronts are numbered level by level (height 0 = leaves first) so that each
// level is a contiguous range and can be processed by one batched launch.
#include "fdfd_internal.h"

#include <algorithm>
#include <cstring>

namespace fdfd {

namespace {

struct Node {
    std::vector<int32_t> S, B;
    int32_t child[2] = {-1, -1};
    int32_t parent = -1;
    int32_t height = 0;
};

struct Builder {
    int32_t Nx, Ny, leaf;
    std::vector<Node> nodes;

    int32_t cell(int32_t i, int32_t j) const { return i * Ny + j; }
    int32_t wi(int32_t i) const { return ((i % Nx) + Nx) % Nx; }
    int32_t wj(int32_t j) const { return ((j % Ny) + Ny) % Ny; }

    // Cells outside [i0,i1)x[j0,j1) that share an edge with it (torus).
    void ring(int32_t i0, int32_t i1, int32_t j0, int32_t j1,
              std::vector<int32_t> &B) const {
        B.clear();
        for (int32_t j = j0; j < j1; ++j) {
            B.push_back(cell(wi(i0 - 1), j));
            B.push_back(cell(wi(i1), j));
        }
        for (int32_t i = i0; i < i1; ++i) {
            B.push_back(cell(i, wj(j0 - 1)));
            B.push_back(cell(i, wj(j1)));
        }
        std::sort(B.begin(), B.end());
        B.erase(std::unique(B.begin(), B.end()), B.end());
        // Drop cells that wrap back inside the rectangle.
        B.erase(std::remove_if(B.begin(), B.end(),
                               [&](int32_t c) {
                                   int32_t i = c / Ny, j = c % Ny;
                                   return i >= i0 && i < i1 && j >= j0 && j < j1;
                               }),
                B.end());
    }

    int32_t add(Node &&nd) {
        int32_t id = (int32_t)nodes.size();
        int32_t h = 0;
        for (int c = 0; c < 2; ++c)
            if (nd.child[c] >= 0) h = std::max(h, nodes[nd.child[c]].height + 1);
        nd.height = h;
        nodes.push_back(std::move(nd));
        for (int c = 0; c < 2; ++c)
            if (nodes[id].child[c] >= 0) nodes[nodes[id].child[c]].parent = id;
        return id;
    }

    int32_t build(int32_t i0, int32_t i1, int32_t j0, int32_t j1) {
        if (i1 <= i0 || j1 <= j0) return -1;
        const int32_t a = i1 - i0, b = j1 - j0;
        Node nd;
        if ((int64_t)a * b <= leaf) {
            for (int32_t i = i0; i < i1; ++i)
                for (int32_t j = j0; j < j1; ++j) nd.S.push_back(cell(i, j));
        } else if (a >= b) {
            const int32_t mid = (i0 + i1) / 2;
            for (int32_t j = j0; j < j1; ++j) nd.S.push_back(cell(mid, j));
            int32_t c0 = build(i0, mid, j0, j1);
            int32_t c1 = build(mid + 1, i1, j0, j1);
            if (c0 < 0) { c0 = c1; c1 = -1; }
            nd.child[0] = c0; nd.child[1] = c1;
        } else {
            const int32_t mid = (j0 + j1) / 2;
            for (int32_t i = i0; i < i1; ++i) nd.S.push_back(cell(i, mid));
            int32_t c0 = build(i0, i1, j0, mid);
            int32_t c1 = build(i0, i1, mid + 1, j1);
            if (c0 < 0) { c0 = c1; c1 = -1; }
            nd.child[0] = c0; nd.child[1] = c1;
        }
        ring(i0, i1, j0, j1, nd.B);
        return add(std::move(nd));
    }
};

inline int64_t sum_sq(int64_t x) { return x <= 0 ? 0 : x * (x + 1) * (2 * x + 1) / 6; }

}  // namespace

int build_symbolic(int32_t Nx, int32_t Ny, int32_t leaf_area, Symbolic &S) {
    if (Nx < 1 || Ny < 1) return fail(FDFD_ERR_BAD_ARG, "symbolic: grid must be at least 1x1");
    if ((int64_t)Nx * Ny > (int64_t)1 << 30)
        return fail(FDFD_ERR_BAD_ARG, "symbolic: grid larger than 2^30 cells");
    if (leaf_area < 1) leaf_area = 1;
    const int32_t n = Nx * Ny;

    Builder bd{Nx, Ny, leaf_area, {}};
    bd.nodes.reserve(2 * (size_t)(n / std::max(1, leaf_area / 2)) + 16);
    int32_t rchild = bd.build(1, Nx, 1, Ny);
    {
        Node root;
        for (int32_t j = 0; j < Ny; ++j) root.S.push_back(bd.cell(0, j));
        for (int32_t i = 1; i < Nx; ++i) root.S.push_back(bd.cell(i, 0));
        root.child[0] = rchild;
        bd.add(std::move(root));
    }
    const int32_t nf = (int32_t)bd.nodes.size();

    // Level order: stable by height (creation order is a postorder).
    std::vector<int32_t> order(nf), newid(nf);
    for (int32_t f = 0; f < nf; ++f) order[f] = f;
    std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) {
        return bd.nodes[a].height < bd.nodes[b].height;
    });
    for (int32_t f = 0; f < nf; ++f) newid[order[f]] = f;

    S = Symbolic();
    S.Nx = Nx; S.Ny = Ny; S.leaf_area = leaf_area; S.nf = nf;
    S.p.resize(nf); S.m.resize(nf); S.ld.resize(nf); S.parent.resize(nf);
    S.child0.resize(nf); S.child1.resize(nf); S.height.resize(nf);
    S.vars_off.resize(nf); S.pool_off.resize(nf);
    int64_t off = 0, poff = 0;
    for (int32_t f = 0; f < nf; ++f) {
        const Node &nd = bd.nodes[order[f]];
        S.p[f] = (int32_t)nd.S.size();
        S.m[f] = (int32_t)(nd.S.size() + nd.B.size());
        S.ld[f] = (S.m[f] + 3) & ~3;
        S.parent[f] = nd.parent >= 0 ? newid[nd.parent] : -1;
        S.child0[f] = nd.child[0] >= 0 ? newid[nd.child[0]] : -1;
        S.child1[f] = nd.child[1] >= 0 ? newid[nd.child[1]] : -1;
        S.height[f] = nd.height;
        if (off > INT32_MAX - S.m[f])
            return fail(FDFD_ERR_BAD_ARG, "symbolic: index lists exceed 2^31 entries");
        S.vars_off[f] = (int32_t)off;
        S.pool_off[f] = poff;
        off += S.m[f];
        poff += (int64_t)S.ld[f] * S.m[f];
    }
    S.sum_m = off;
    S.pool_entries = poff;
    S.vars.resize(off);
    S.relmap.assign(off, -1);
    for (int32_t f = 0; f < nf; ++f) {
        const Node &nd = bd.nodes[order[f]];
        int32_t *v = S.vars.data() + S.vars_off[f];
        std::memcpy(v, nd.S.data(), nd.S.size() * sizeof(int32_t));
        std::memcpy(v + nd.S.size(), nd.B.data(), nd.B.size() * sizeof(int32_t));
    }
    bd.nodes.clear();
    bd.nodes.shrink_to_fit();

    // Levels.
    S.nlev = nf ? S.height[nf - 1] + 1 : 0;
    S.level_ptr.assign(S.nlev + 1, 0);
    for (int32_t f = 0; f < nf; ++f) S.level_ptr[S.height[f] + 1]++;
    for (int32_t L = 0; L < S.nlev; ++L) S.level_ptr[L + 1] += S.level_ptr[L];
    S.lev_max_m.assign(S.nlev, 0);
    S.lev_max_p.assign(S.nlev, 0);

    // Index maps.
    S.var_front.assign(n, -1);
    S.var_loc.assign(n, -1);
    S.nbr_loc.assign((size_t)4 * n, -1);
    std::vector<int32_t> pos(n, -1);
    for (int32_t f = 0; f < nf; ++f) {
        const int32_t m = S.m[f], p = S.p[f];
        const int32_t *v = S.vars.data() + S.vars_off[f];
        for (int32_t k = 0; k < m; ++k) {
            if (pos[v[k]] >= 0)
                return fail(FDFD_ERR_BAD_ARG, "symbolic: duplicate variable in a front");
            pos[v[k]] = k;
        }
        for (int32_t k = 0; k < p; ++k) {
            const int32_t s = v[k];
            if (S.var_front[s] >= 0)
                return fail(FDFD_ERR_BAD_ARG, "symbolic: variable eliminated twice");
            S.var_front[s] = f;
            S.var_loc[s] = k;
            const int32_t i = s / Ny, j = s % Ny;
            const int32_t nb[4] = {((i - 1 + Nx) % Nx) * Ny + j, ((i + 1) % Nx) * Ny + j,
                                   i * Ny + (j - 1 + Ny) % Ny, i * Ny + (j + 1) % Ny};
            for (int d = 0; d < 4; ++d) S.nbr_loc[(size_t)4 * s + d] = pos[nb[d]];
        }
        const int32_t ch[2] = {S.child0[f], S.child1[f]};
        for (int c = 0; c < 2; ++c) {
            if (ch[c] < 0) continue;
            const int32_t cm = S.m[ch[c]], cp = S.p[ch[c]];
            const int32_t *cv = S.vars.data() + S.vars_off[ch[c]];
            int32_t *rm = S.relmap.data() + S.vars_off[ch[c]];
            for (int32_t k = cp; k < cm; ++k) {
                if (pos[cv[k]] < 0)
                    return fail(FDFD_ERR_BAD_ARG, "symbolic: child boundary not in parent front");
                rm[k] = pos[cv[k]];
            }
        }
        for (int32_t k = 0; k < m; ++k) pos[v[k]] = -1;

        const int32_t L = S.height[f];
        S.lev_max_m[L] = std::max(S.lev_max_m[L], m);
        S.lev_max_p[L] = std::max(S.lev_max_p[L], p);
        S.max_m = std::max(S.max_m, m);
        S.max_p = std::max(S.max_p, p);
        S.factor_entries += (int64_t)p * p + 2 * (int64_t)p * (m - p);
        S.factor_flops += 8.0 * (double)(sum_sq(m - 1) - sum_sq(m - p - 1));
    }
    for (int32_t s = 0; s < n; ++s)
        if (S.var_front[s] < 0) return fail(FDFD_ERR_BAD_ARG, "symbolic: variable never eliminated");
    S.rows = Nx;
    return FDFD_OK;
}

// The forest of `batch` copies of one tree.  Copy b of front f of level L
// gets the id level_ptr'[L] + b * cnt_L + (f - level_ptr[L]) (a level's
// copies are contiguous, so one launch per level still covers every front
// of every problem); copy b's variables are the single tree's plus b * n.
int replicate_symbolic(const Symbolic &S1, int32_t batch, Symbolic &S) {
    if (batch < 1) return fail(FDFD_ERR_BAD_ARG, "symbolic: batch must be >= 1");
    const int64_t n1 = (int64_t)S1.Nx * S1.Ny;
    if (n1 * batch > ((int64_t)1 << 30) / 5 || S1.sum_m * batch > INT32_MAX)
        return fail(FDFD_ERR_BAD_ARG, "symbolic: batch too large for int32 indices");
    const int32_t nf1 = S1.nf, nlev = S1.nlev;
    S = Symbolic();
    S.batch = batch;
    S.rows = S1.Nx;
    S.Nx = S1.Nx * batch;
    S.Ny = S1.Ny;
    S.leaf_area = S1.leaf_area;
    S.nf = nf1 * batch;
    S.nlev = nlev;
    S.level_ptr.assign(nlev + 1, 0);
    for (int32_t L = 0; L < nlev; ++L)
        S.level_ptr[L + 1] = S.level_ptr[L] + batch * (S1.level_ptr[L + 1] - S1.level_ptr[L]);
    auto nid = [&](int32_t b, int32_t f) -> int32_t {
        if (f < 0) return -1;
        const int32_t L = S1.height[f], cnt = S1.level_ptr[L + 1] - S1.level_ptr[L];
        return S.level_ptr[L] + b * cnt + (f - S1.level_ptr[L]);
    };
    const int32_t nf = S.nf;
    S.p.resize(nf); S.m.resize(nf); S.ld.resize(nf); S.parent.resize(nf);
    S.child0.resize(nf); S.child1.resize(nf); S.height.resize(nf);
    S.vars_off.resize(nf); S.pool_off.resize(nf);
    std::vector<int32_t> src(nf), prob(nf);
    for (int32_t b = 0; b < batch; ++b)
        for (int32_t f = 0; f < nf1; ++f) {
            const int32_t g = nid(b, f);
            src[g] = f;
            prob[g] = b;
            S.p[g] = S1.p[f]; S.m[g] = S1.m[f]; S.ld[g] = S1.ld[f]; S.height[g] = S1.height[f];
            S.parent[g] = nid(b, S1.parent[f]);
            S.child0[g] = nid(b, S1.child0[f]);
            S.child1[g] = nid(b, S1.child1[f]);
        }
    int64_t off = 0, poff = 0;
    for (int32_t g = 0; g < nf; ++g) {
        S.vars_off[g] = (int32_t)off;
        S.pool_off[g] = poff;
        off += S.m[g];
        poff += (int64_t)S.ld[g] * S.m[g];
    }
    S.sum_m = off;
    S.pool_entries = poff;
    S.vars.resize(off);
    S.relmap.resize(off);
    for (int32_t g = 0; g < nf; ++g) {
        const int32_t f = src[g], m = S.m[g];
        const int32_t add = (int32_t)(prob[g] * n1);
        const int32_t *v1 = S1.vars.data() + S1.vars_off[f];
        const int32_t *r1 = S1.relmap.data() + S1.vars_off[f];
        int32_t *v = S.vars.data() + S.vars_off[g];
        int32_t *r = S.relmap.data() + S.vars_off[g];
        for (int32_t k = 0; k < m; ++k) {
            v[k] = v1[k] + add;
            r[k] = r1[k];
        }
    }
    const int64_t n = n1 * batch;
    S.var_front.resize(n);
    S.var_loc.resize(n);
    S.nbr_loc.resize((size_t)4 * n);
    for (int32_t b = 0; b < batch; ++b)
        for (int64_t s = 0; s < n1; ++s) {
            S.var_front[b * n1 + s] = nid(b, S1.var_front[s]);
            S.var_loc[b * n1 + s] = S1.var_loc[s];
            for (int d = 0; d < 4; ++d) S.nbr_loc[(size_t)4 * (b * n1 + s) + d] = S1.nbr_loc[(size_t)4 * s + d];
        }
    S.lev_max_m = S1.lev_max_m;
    S.lev_max_p = S1.lev_max_p;
    S.factor_entries = S1.factor_entries * batch;
    S.factor_flops = S1.factor_flops * batch;
    S.max_m = S1.max_m;
    S.max_p = S1.max_p;
    return FDFD_OK;
}

}  // namespace fdfd

// ---- C ABI ---------------------------------------------------------------
using fdfd::fail;

extern "C" int fdfd_symbolic_create(int32_t Nx, int32_t Ny, int32_t leaf_area,
                                    fdfd_symbolic **out) {
    if (!out) return fail(FDFD_ERR_BAD_ARG, "symbolic_create: out is NULL");
    *out = nullptr;
    fdfd_symbolic *h = nullptr;
    try {
        h = new fdfd_symbolic();
        int st = fdfd::build_symbolic(Nx, Ny, leaf_area, h->s);
        if (st != FDFD_OK) { delete h; return st; }
    } catch (const std::bad_alloc &) {
        delete h;
        return fail(FDFD_ERR_OOM, "symbolic_create: host allocation failed");
    }
    *out = h;
    return FDFD_OK;
}

extern "C" int fdfd_symbolic_create_batch(int32_t Nx, int32_t Ny, int32_t leaf_area, int32_t batch,
                                          fdfd_symbolic **out) {
    if (!out) return fail(FDFD_ERR_BAD_ARG, "symbolic_create_batch: out is NULL");
    *out = nullptr;
    fdfd_symbolic *h = nullptr;
    try {
        fdfd::Symbolic one;
        int st = fdfd::build_symbolic(Nx, Ny, leaf_area, one);
        if (st != FDFD_OK) return st;
        h = new fdfd_symbolic();
        st = fdfd::replicate_symbolic(one, batch, h->s);
        if (st != FDFD_OK) { delete h; return st; }
    } catch (const std::bad_alloc &) {
        delete h;
        return fail(FDFD_ERR_OOM, "symbolic_create_batch: host allocation failed");
    }
    *out = h;
    return FDFD_OK;
}

extern "C" int fdfd_symbolic_info_get(const fdfd_symbolic *sym, fdfd_symbolic_info *info) {
    if (!sym || !info) return fail(FDFD_ERR_BAD_ARG, "symbolic_info: NULL argument");
    const fdfd::Symbolic &S = sym->s;
    info->Nx = S.Nx; info->Ny = S.Ny;
    info->n_fronts = S.nf; info->n_levels = S.nlev;
    info->sum_m = S.sum_m; info->pool_entries = S.pool_entries;
    info->factor_entries = S.factor_entries; info->factor_flops = S.factor_flops;
    info->max_m = S.max_m; info->max_p = S.max_p;
    return FDFD_OK;
}

extern "C" int fdfd_symbolic_export(const fdfd_symbolic *sym, int32_t which, void *dst) {
    if (!sym || !dst) return fail(FDFD_ERR_BAD_ARG, "symbolic_export: NULL argument");
    const fdfd::Symbolic &S = sym->s;
    const std::vector<int32_t> *v32 = nullptr;
    switch (which) {
        case 0: v32 = &S.p; break;
        case 1: v32 = &S.m; break;
        case 2: v32 = &S.parent; break;
        case 3: v32 = &S.child0; break;
        case 4: v32 = &S.child1; break;
        case 5: v32 = &S.height; break;
        case 6: v32 = &S.vars_off; break;
        case 7: v32 = &S.level_ptr; break;
        case 8: v32 = &S.vars; break;
        case 9: v32 = &S.relmap; break;
        case 10: v32 = &S.nbr_loc; break;
        case 11: v32 = &S.var_front; break;
        case 12: v32 = &S.var_loc; break;
        case 13: v32 = &S.ld; break;
        case 14:
            std::memcpy(dst, S.pool_off.data(), S.pool_off.size() * sizeof(int64_t));
            return FDFD_OK;
        default: return fail(FDFD_ERR_BAD_ARG, "symbolic_export: unknown array id");
    }
    std::memcpy(dst, v32->data(), v32->size() * sizeof(int32_t));
    return FDFD_OK;
}

extern "C" void fdfd_symbolic_destroy(fdfd_symbolic *sym) { delete sym; }
