// plan.cpp -- per-dataset pair plan: column-pattern compression, unique pair
// lists per tree node, child gather indices, level schedule and partial-buffer
// arena layout.
//
// Semantics follow getindexdict (src/FelsensteinCUDA.jl:77-142) and
// Dataset.subcolumnrefs (src/Dataset.jl:180-196): at node v two root pairs
// share one partial when their columns have the same subtree patterns at v.
// The set of unique pairs at v is derived from the parent's unique list, so
// every node computes each distinct (pattern_v(x), pattern_v(y)) exactly
// once.  Results do not depend on the dedup, only the work does.
#include <algorithm>
#include <cstring>

#include "internal.h"

namespace messi {

namespace {

// Open-addressing int64 -> int32 map.
struct KeyMap {
    std::vector<int64_t> keys;
    std::vector<int32_t> vals;
    uint64_t mask = 0;
    void reset(size_t expected)
    {
        size_t cap = 16;
        while (cap < 2 * expected + 2) cap <<= 1;
        keys.assign(cap, -1);
        vals.resize(cap);
        mask = cap - 1;
    }
    // Returns the value for key, inserting `next` if absent (then *inserted = true).
    int32_t get_or_insert(int64_t key, int32_t next, bool* inserted)
    {
        uint64_t h = ((uint64_t)key * 0x9E3779B97F4A7C15ull) >> 20;
        uint64_t s = h & mask;
        while (keys[s] >= 0 && keys[s] != key) s = (s + 1) & mask;
        if (keys[s] < 0) {
            keys[s] = key;
            vals[s] = next;
            *inserted = true;
            return next;
        }
        *inserted = false;
        return vals[s];
    }
};

}  // namespace

int build_plan(messi_dataset* ds, const messi_alignment* aln, int W, const uint8_t* pairmask, std::string* err,
               const std::vector<int2>* pairs, std::vector<int32_t>* pair_unique)
{
    const int N = aln->numseqs, L = aln->numcols, nn = aln->numnodes;
    if (N < 2 || L < 1 || nn != 2 * N - 1 || !aln->masks || !aln->children || !aln->seqindex) {
        *err = "alignment: need numseqs >= 2, numcols >= 1, numnodes == 2*numseqs-1 and all arrays";
        return MESSI_EINVAL;
    }
    if (W < 1) W = 1;
    if (W > L - 1) W = (L > 1) ? L - 1 : 1;
    ds->N = N;
    ds->L = L;
    ds->numnodes = nn;
    ds->W = W;
    ds->children.assign(aln->children, aln->children + 2 * nn);
    ds->seqindex.assign(aln->seqindex, aln->seqindex + nn);
    ds->masks.assign(aln->masks, aln->masks + (size_t)N * L);
    for (size_t i = 0; i < ds->masks.size(); i++)
        if (ds->masks[i] == 0 || ds->masks[i] > 15) {
            *err = "alignment: nucleotide masks must be in 1..15";
            return MESSI_EINVAL;
        }
    // ---- validate the tree: binary, pre-order numbering, every node reached once
    ds->parent.assign(nn, -1);
    std::vector<int> seen_seq(N, 0);
    for (int v = 0; v < nn; v++) {
        int c0 = ds->children[2 * v], c1 = ds->children[2 * v + 1];
        if ((c0 < 0) != (c1 < 0)) { *err = "tree: every internal node needs two children"; return MESSI_EINVAL; }
        if (c0 < 0) {
            int s = ds->seqindex[v];
            if (s < 0 || s >= N || seen_seq[s]) { *err = "tree: leaves must map one-to-one to sequences"; return MESSI_EINVAL; }
            seen_seq[s] = 1;
        } else {
            for (int c : {c0, c1}) {
                if (c <= v || c >= nn || ds->parent[c] >= 0) {
                    *err = "tree: children must be later pre-order nodes with a single parent";
                    return MESSI_EINVAL;
                }
                ds->parent[c] = v;
            }
        }
    }
    for (int v = 1; v < nn; v++)
        if (ds->parent[v] < 0) { *err = "tree: node not reachable from the root"; return MESSI_EINVAL; }
    // post-order and levels
    ds->postorder.clear();
    {
        std::vector<int> stack{0};
        std::vector<char> expanded(nn, 0);
        while (!stack.empty()) {
            int v = stack.back();
            if (ds->children[2 * v] < 0 || expanded[v]) {
                ds->postorder.push_back(v);
                stack.pop_back();
            } else {
                expanded[v] = 1;
                stack.push_back(ds->children[2 * v + 1]);
                stack.push_back(ds->children[2 * v]);
            }
        }
    }
    ds->level.assign(nn, 0);
    int maxdepth = 0;
    {
        std::vector<int> depth(nn, 0);
        for (int v = 1; v < nn; v++) depth[v] = depth[ds->parent[v]] + 1;  // parent < v
        for (int v = 0; v < nn; v++) maxdepth = std::max(maxdepth, depth[v]);
    }
    if (maxdepth + 2 > kMaxStack) { *err = "tree: height above the supported limit (510)"; return MESSI_EINVAL; }
    for (int v : ds->postorder)
        if (ds->children[2 * v] >= 0)
            ds->level[v] = 1 + std::max(ds->level[ds->children[2 * v]], ds->level[ds->children[2 * v + 1]]);
    ds->H = ds->level[0];

    // ---- column pattern ids per node (dense, first-occurrence order)
    std::vector<std::vector<int32_t>> pid(nn);
    std::vector<int32_t> npat(nn, 0);
    KeyMap km;
    for (int v : ds->postorder) {
        pid[v].resize(L);
        if (ds->children[2 * v] < 0) {
            int first[16];
            for (int k = 0; k < 16; k++) first[k] = -1;
            const uint8_t* row = &ds->masks[(size_t)ds->seqindex[v] * L];
            int n = 0;
            for (int x = 0; x < L; x++) {
                if (first[row[x]] < 0) first[row[x]] = n++;
                pid[v][x] = first[row[x]];
            }
            npat[v] = n;
        } else {
            int c0 = ds->children[2 * v], c1 = ds->children[2 * v + 1];
            km.reset(std::min<size_t>((size_t)L, (size_t)npat[c0] * npat[c1]));
            int n = 0;
            for (int x = 0; x < L; x++) {
                bool ins;
                int64_t key = (int64_t)pid[c0][x] * npat[c1] + pid[c1][x];
                pid[v][x] = km.get_or_insert(key, n, &ins);
                if (ins) n++;
            }
            npat[v] = n;
        }
    }

    // ---- unique pairs at the root (band + mask, or an explicit pair list), band index map
    const int W1 = W + 1;
    std::vector<int32_t> bandidx(pairs ? (size_t)1 : (size_t)L * W1, -1);
    std::vector<std::vector<int32_t>> rep(nn);  // representative (x, y) per unique pair, interleaved
    ds->nunique.assign(nn, 0);
    if (pairs) {
        ds->band_pairs = (int64_t)pairs->size();
        km.reset((size_t)std::min<int64_t>(ds->band_pairs, (int64_t)npat[0] * npat[0]));
        pair_unique->assign(pairs->size(), -1);
        int32_t n = 0;
        for (size_t p = 0; p < pairs->size(); p++) {
            const int x = (*pairs)[p].x, y = (*pairs)[p].y;
            if (x < 0 || y >= L || x >= y) {
                *err = "structure: pairs must satisfy 0 <= x < y < numcols";
                return MESSI_EINVAL;
            }
            bool ins;
            const int64_t key = (int64_t)pid[0][x] * npat[0] + pid[0][y];
            const int32_t u = km.get_or_insert(key, n, &ins);
            if (ins) {
                rep[0].push_back(x);
                rep[0].push_back(y);
                n++;
            }
            (*pair_unique)[p] = u;
        }
        ds->nroot = n;
        ds->nunique[0] = n;
    } else {
        int64_t count_band = 0;
        for (int x = 0; x < L; x++) {
            int kmax = std::min(W, L - 1 - x);
            for (int k = 1; k <= kmax; k++)
                if (!pairmask || pairmask[(size_t)x + (size_t)(x + k) * L]) count_band++;
        }
        ds->band_pairs = count_band;
        km.reset((size_t)std::min<int64_t>(count_band, (int64_t)npat[0] * npat[0]));
        int32_t n = 0;
        for (int x = 0; x < L; x++) {
            int kmax = std::min(W, L - 1 - x);
            for (int k = 1; k <= kmax; k++) {
                int y = x + k;
                if (pairmask && !pairmask[(size_t)x + (size_t)y * L]) continue;
                bool ins;
                int64_t key = (int64_t)pid[0][x] * npat[0] + pid[0][y];
                int32_t u = km.get_or_insert(key, n, &ins);
                if (ins) {
                    rep[0].push_back(x);
                    rep[0].push_back(y);
                    n++;
                }
                bandidx[(size_t)x * W1 + k] = u;
            }
        }
        ds->nroot = n;
        ds->nunique[0] = n;
    }

    // ---- unique pairs per node from the parent's list (pre-order: parents first)
    std::vector<std::vector<int32_t>> li(nn), ri(nn);
    for (int v = 0; v < nn; v++) {
        if (ds->children[2 * v] < 0) continue;
        const int64_t nv = ds->nunique[v];
        for (int side = 0; side < 2; side++) {
            int c = ds->children[2 * v + side];
            std::vector<int32_t>& idx = side ? ri[v] : li[v];
            idx.resize(nv);
            km.reset((size_t)std::min<int64_t>(nv, (int64_t)npat[c] * npat[c]));
            int32_t n = 0;
            for (int64_t u = 0; u < nv; u++) {
                int x = rep[v][2 * u], y = rep[v][2 * u + 1];
                bool ins;
                int64_t key = (int64_t)pid[c][x] * npat[c] + pid[c][y];
                int32_t cu = km.get_or_insert(key, n, &ins);
                if (ins) {
                    rep[c].push_back(x);
                    rep[c].push_back(y);
                    n++;
                }
                idx[u] = cu;
            }
            ds->nunique[c] = n;
        }
        if (v != 0) { std::vector<int32_t>().swap(rep[v]); }
    }

    // ---- statistics
    ds->executed = 0;
    for (int v = 0; v < nn; v++)
        if (ds->children[2 * v] >= 0) ds->executed += ds->nunique[v];
    ds->naive = ds->band_pairs * (int64_t)(N - 1);

    // ---- leaf tables: row u = outer product of the two column masks
    ds->leaf_off.assign(nn, -1);
    int64_t leaf_rows = 0;
    for (int v = 0; v < nn; v++)
        if (ds->children[2 * v] < 0) { ds->leaf_off[v] = leaf_rows; leaf_rows += ds->nunique[v]; }
    ds->leaf_rows = leaf_rows;
    std::vector<float>& leaf = ds->leaf_host;
    leaf.assign((size_t)std::max<int64_t>(leaf_rows, 1) * 16, 0.f);
    ds->leafnode_host.assign((size_t)std::max<int64_t>(leaf_rows, 1), 0);
    for (int v = 0; v < nn; v++) {
        if (ds->children[2 * v] >= 0) continue;
        const uint8_t* row = &ds->masks[(size_t)ds->seqindex[v] * L];
        for (int64_t u = 0; u < ds->nunique[v]; u++) {
            uint8_t mx = row[rep[v][2 * u]], my = row[rep[v][2 * u + 1]];
            float* o = &leaf[(size_t)(ds->leaf_off[v] + u) * 16];
            for (int a = 0; a < 16; a++) o[a] = (float)(((mx >> (a / 4)) & 1) * ((my >> (a % 4)) & 1));
            ds->leafnode_host[ds->leaf_off[v] + u] = v;
        }
    }

    // ---- arena layout over levels: a node's rows live from its level to its parent's
    ds->row_off.assign(nn, -1);
    ds->level_nodes.assign(ds->H + 1, {});
    for (int v = 0; v < nn; v++)
        if (ds->children[2 * v] >= 0) ds->level_nodes[ds->level[v]].push_back(v);
    {
        struct Iv { int64_t off, len; int node; };
        std::vector<Iv> live;
        int64_t peak = 0;
        for (int lv = 1; lv <= ds->H; lv++) {
            live.erase(std::remove_if(live.begin(), live.end(),
                                      [&](const Iv& iv) { return ds->level[ds->parent[iv.node]] < lv; }),
                       live.end());
            for (int v : ds->level_nodes[lv]) {
                if (v == 0) continue;  // the root writes mixtures, not rows
                int64_t len = ds->nunique[v];
                std::sort(live.begin(), live.end(), [](const Iv& a, const Iv& b) { return a.off < b.off; });
                int64_t pos = 0;
                for (const Iv& iv : live) {
                    if (iv.off - pos >= len) break;
                    pos = std::max(pos, iv.off + iv.len);
                }
                live.push_back({pos, len, v});
                ds->row_off[v] = pos;
                peak = std::max(peak, pos + len);
            }
        }
        ds->arena_rows = std::max<int64_t>(peak, 1);
    }

    // ---- upload static device data
    cudaError_t e;
    int64_t lr_total = 0;
    ds->lr_off.assign(nn, -1);
    for (int v = 0; v < nn; v++)
        if (ds->children[2 * v] >= 0) { ds->lr_off[v] = lr_total; lr_total += 2 * ds->nunique[v]; }
    std::vector<int32_t> lr((size_t)std::max<int64_t>(lr_total, 1));
    for (int v = 0; v < nn; v++)
        if (ds->children[2 * v] >= 0) {
            std::copy(li[v].begin(), li[v].end(), lr.begin() + ds->lr_off[v]);
            std::copy(ri[v].begin(), ri[v].end(), lr.begin() + ds->lr_off[v] + ds->nunique[v]);
        }
    std::vector<int> tree((size_t)nn * 4);
    for (int v = 0; v < nn; v++) {
        tree[4 * v] = ds->children[2 * v];
        tree[4 * v + 1] = ds->children[2 * v + 1];
        tree[4 * v + 2] = ds->seqindex[v];
        tree[4 * v + 3] = 0;
    }
#define UPLOAD(dst, src, bytes)                                                       \
    do {                                                                              \
        if ((e = cudaMalloc((void**)&(dst), (bytes))) != cudaSuccess) goto cuda_error; \
        if ((e = cudaMemcpy((dst), (src), (bytes), cudaMemcpyHostToDevice)) != cudaSuccess) goto cuda_error; \
    } while (0)
    UPLOAD(ds->d_bandidx, bandidx.data(), bandidx.size() * sizeof(int32_t));
    UPLOAD(ds->d_lr, lr.data(), lr.size() * sizeof(int32_t));
    UPLOAD(ds->d_leaf, leaf.data(), leaf.size() * sizeof(float));
    UPLOAD(ds->d_leafnode, ds->leafnode_host.data(), ds->leafnode_host.size() * sizeof(int));
    UPLOAD(ds->d_masks, ds->masks.data(), ds->masks.size());
    UPLOAD(ds->d_tree, tree.data(), tree.size() * sizeof(int));
    UPLOAD(ds->d_post, ds->postorder.data(), ds->postorder.size() * sizeof(int));
#undef UPLOAD
    if ((e = cudaMalloc((void**)&ds->d_mix, sizeof(double) * std::max<int64_t>(ds->nroot, 1))) != cudaSuccess)
        goto cuda_error;
    if ((e = cudaMalloc((void**)&ds->d_mixlam, sizeof(double) * kMaxLambda * std::max<int64_t>(ds->nroot, 1))) !=
        cudaSuccess)
        goto cuda_error;
    {
        // tiles per level
        std::vector<int2> tiles;
        ds->tile_off.assign(ds->H + 1, 0);
        ds->tile_cnt.assign(ds->H + 1, 0);
        for (int lv = 1; lv <= ds->H; lv++) {
            ds->tile_off[lv] = (int)tiles.size();
            for (int v : ds->level_nodes[lv])
                for (int64_t b = 0; b < ds->nunique[v]; b += kTile) tiles.push_back(make_int2(v, (int)b));
            ds->tile_cnt[lv] = (int)tiles.size() - ds->tile_off[lv];
        }
        if (tiles.empty()) tiles.push_back(make_int2(0, 0));
        if ((e = cudaMalloc((void**)&ds->d_tiles, tiles.size() * sizeof(int2))) != cudaSuccess) goto cuda_error;
        if ((e = cudaMemcpy(ds->d_tiles, tiles.data(), tiles.size() * sizeof(int2), cudaMemcpyHostToDevice)) !=
            cudaSuccess)
            goto cuda_error;
        if ((e = cudaMalloc((void**)&ds->d_nodes, sizeof(NodeDev) * nn)) != cudaSuccess) goto cuda_error;
    }
    return MESSI_OK;
cuda_error:
    *err = std::string("dataset upload: ") + cudaGetErrorString(e);
    return (e == cudaErrorMemoryAllocation) ? MESSI_ENOMEM : MESSI_ECUDA;
}

void fill_node_descriptors(const messi_dataset* ds, float* arena_f, int* arena_e, int64_t row_base, int64_t cstride,
                           float* leafmsg, int64_t leaf_base, int64_t leaf_cstride, int node_base, int grp,
                           NodeDev* out)
{
    for (int v = 0; v < ds->numnodes; v++) {
        NodeDev& d = out[v];
        d = NodeDev{};
        if (ds->children[2 * v] < 0) continue;
        d.n = (int)ds->nunique[v];
        d.li = ds->d_lr + ds->lr_off[v];
        d.ri = ds->d_lr + ds->lr_off[v] + ds->nunique[v];
        const int c0 = ds->children[2 * v], c1 = ds->children[2 * v + 1];
        d.self = node_base + v;
        d.grp = grp;
        for (int side = 0; side < 2; side++) {
            const int c = side ? c1 : c0;
            const float* f;
            const int* ex;
            long long cs;
            if (ds->children[2 * c] < 0) {
                f = leafmsg + (size_t)(leaf_base + ds->leaf_off[c]) * 16;
                ex = nullptr;
                cs = leaf_cstride;
            } else {
                f = arena_f + (size_t)(row_base + ds->row_off[c]) * 16;
                ex = arena_e + row_base + ds->row_off[c];
                cs = cstride;
            }
            if (side) { d.rf = f; d.re = ex; d.rcs = cs; }
            else { d.lf = f; d.le = ex; d.lcs = cs; }
        }
        if (v != 0) {
            d.of = arena_f + (size_t)(row_base + ds->row_off[v]) * 16;
            d.oe = arena_e + row_base + ds->row_off[v];
            d.ocs = cstride;
        } else {
            d.mix = ds->d_mix;
            d.mixlam = ds->d_mixlam;
        }
    }
}

// Allocate the partial-row arena for C categories (as many per pass as fit)
// and fill the node descriptors.
int allocate_arena(messi_dataset* ds, int C, std::string* err)
{
    size_t freeb = 0, totalb = 0;
    cudaMemGetInfo(&freeb, &totalb);
    const size_t row_bytes = 16 * sizeof(float) + sizeof(int);
    size_t budget = freeb / 2;
    const int64_t leaf_rows = std::max<int64_t>(ds->leaf_rows, 1);
    int chunk = C;
    while (chunk > 1 && (size_t)chunk * (ds->arena_rows + leaf_rows) * row_bytes > budget) chunk = (chunk + 1) / 2;
    if (ds->chunk != chunk) {
        if (ds->d_arena_f) cudaFree(ds->d_arena_f);
        if (ds->d_arena_e) cudaFree(ds->d_arena_e);
        if (ds->d_leafmsg) cudaFree(ds->d_leafmsg);
        ds->d_arena_f = nullptr;
        ds->d_arena_e = nullptr;
        ds->d_leafmsg = nullptr;
        ds->chunk = 0;
        cudaError_t e = cudaMalloc((void**)&ds->d_arena_f, (size_t)chunk * ds->arena_rows * 16 * sizeof(float));
        if (e == cudaSuccess) e = cudaMalloc((void**)&ds->d_arena_e, (size_t)chunk * ds->arena_rows * sizeof(int));
        if (e == cudaSuccess) e = cudaMalloc((void**)&ds->d_leafmsg, (size_t)chunk * leaf_rows * 16 * sizeof(float));
        if (e != cudaSuccess) {
            *err = std::string("message arena: ") + cudaGetErrorString(e);
            return MESSI_ENOMEM;
        }
        ds->chunk = chunk;
    }
    ds->arena_gen++;
    ds->nodes_host.assign(ds->numnodes, NodeDev{});
    fill_node_descriptors(ds, ds->d_arena_f, ds->d_arena_e, 0, ds->arena_rows, ds->d_leafmsg, 0, leaf_rows, 0, 0,
                          ds->nodes_host.data());
    const int nn = ds->numnodes;
    cudaError_t e = cudaMemcpy(ds->d_nodes, ds->nodes_host.data(), sizeof(NodeDev) * nn, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        *err = std::string("node descriptors: ") + cudaGetErrorString(e);
        return MESSI_ECUDA;
    }
    return MESSI_OK;
}

}  // namespace messi
