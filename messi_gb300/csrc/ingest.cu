// ingest.cu -- column-pattern compression on the device.
//
// Replaces the Dict loop of the Dataset constructor that builds
// subcolumnrefs (src/Dataset.jl:180-196): for every tree node v and column
// x, the first column whose subtree pattern at v equals that of x.  The
// pattern at a leaf is the column's nucleotide mask; at an internal node it
// is the pair (pattern at child 0, pattern at child 1), and the first-column
// index of a pattern identifies it, so the key of (v, x) is
// refs[c0][x] * L + refs[c1][x].  Nodes are processed level by level from the
// leaves; per node an open-addressing table keeps, for each key, the
// smallest column (atomicMin), and a lookup pass writes it back.  The result
// is exact (keys are stored, not hashed away).
#include <climits>

#include "internal.h"

namespace messi {

namespace {

constexpr unsigned long long kEmptyKey = ~0ull;

__device__ __forceinline__ unsigned long long pattern_key(const uint8_t* __restrict__ masks,
                                                          const int* __restrict__ tree, const int* __restrict__ refs,
                                                          int v, int x, int L)
{
    const int c0 = tree[4 * v], c1 = tree[4 * v + 1];
    if (c0 < 0) return (unsigned long long)masks[(size_t)tree[4 * v + 2] * L + x];
    return (unsigned long long)refs[(size_t)c0 * L + x] * (unsigned long long)L + (unsigned long long)refs[(size_t)c1 * L + x];
}

__device__ __forceinline__ unsigned int slot_of(unsigned long long key, unsigned int mask)
{
    key ^= key >> 33;
    key *= 0xff51afd7ed558ccdull;
    key ^= key >> 33;
    return (unsigned int)key & mask;
}

}  // namespace

// One launch per tree level: every (node of the level, column) inserts its
// key into the node's table and keeps the smallest column.
__global__ void refs_insert_kernel(const int* __restrict__ level_nodes, const uint8_t* __restrict__ masks,
                                   const int* __restrict__ tree, const int* __restrict__ refs, int L,
                                   unsigned long long* __restrict__ tkeys, int* __restrict__ tvals, int tsize)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= L) return;
    const int v = level_nodes[blockIdx.y];
    const unsigned long long key = pattern_key(masks, tree, refs, v, x, L);
    unsigned long long* keys = tkeys + (size_t)blockIdx.y * tsize;
    int* vals = tvals + (size_t)blockIdx.y * tsize;
    const unsigned int mask = (unsigned int)tsize - 1u;
    unsigned int s = slot_of(key, mask);
    for (int probe = 0; probe < tsize; probe++) {  // at most L keys in 2L+ slots: always ends
        const unsigned long long prev = atomicCAS(&keys[s], kEmptyKey, key);
        if (prev == kEmptyKey || prev == key) {
            atomicMin(&vals[s], x);
            return;
        }
        s = (s + 1u) & mask;
    }
}

// out: the Julia matrix subcolumnrefs[node, col] (column-major, 1-based values)
// when out_julia, else refs only.
__global__ void refs_lookup_kernel(const int* __restrict__ level_nodes, const uint8_t* __restrict__ masks,
                                   const int* __restrict__ tree, int* __restrict__ refs, int L, int numnodes,
                                   const unsigned long long* __restrict__ tkeys, const int* __restrict__ tvals,
                                   int tsize, int* __restrict__ out_julia)
{
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= L) return;
    const int v = level_nodes[blockIdx.y];
    const unsigned long long key = pattern_key(masks, tree, refs, v, x, L);
    const unsigned long long* keys = tkeys + (size_t)blockIdx.y * tsize;
    const int* vals = tvals + (size_t)blockIdx.y * tsize;
    const unsigned int mask = (unsigned int)tsize - 1u;
    unsigned int s = slot_of(key, mask);
    int first = x;
    for (int probe = 0; probe < tsize; probe++) {
        if (keys[s] == key) {
            first = vals[s];
            break;
        }
        s = (s + 1u) & mask;
    }
    refs[(size_t)v * L + x] = first;
    if (out_julia) out_julia[(size_t)v + (size_t)x * numnodes] = first + 1;
}

__global__ void refs_reset_kernel(unsigned long long* __restrict__ tkeys, int* __restrict__ tvals, long long n)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        tkeys[i] = kEmptyKey;
        tvals[i] = INT_MAX;
    }
}

int run_subcolumnrefs(messi_ctx* ctx, messi_dataset* ds, int* d_refs, int* d_out_julia, void* d_work,
                      size_t work_bytes)
{
    const int L = ds->L, nn = ds->numnodes;
    int tsize = 16;
    while (tsize < 2 * L + 2) tsize <<= 1;
    // levels from the leaves (level 0) up; a node's children are at lower levels
    std::vector<std::vector<int>> levels(ds->H + 1);
    for (int v = 0; v < nn; v++) levels[ds->children[2 * v] < 0 ? 0 : ds->level[v]].push_back(v);
    size_t maxw = 1;
    for (const auto& lv : levels) maxw = std::max(maxw, lv.size());
    const size_t need = maxw * tsize * (sizeof(unsigned long long) + sizeof(int)) + (size_t)nn * sizeof(int);
    if (work_bytes < need) return fail(ctx, MESSI_EINVAL, "subcolumnrefs: work buffer too small");
    unsigned long long* tkeys = (unsigned long long*)d_work;
    int* tvals = (int*)(tkeys + maxw * tsize);
    int* d_lv = tvals + maxw * tsize;
    // all level lists in one upload
    std::vector<int> flat;
    std::vector<size_t> off;
    for (const auto& lv : levels) {
        off.push_back(flat.size());
        flat.insert(flat.end(), lv.begin(), lv.end());
    }
    int rc = h2d(ctx, d_lv, flat.data(), flat.size() * sizeof(int));
    if (rc) return rc;
    const int bs = 256;
    for (size_t l = 0; l < levels.size(); l++) {
        const int cnt = (int)levels[l].size();
        if (cnt == 0) continue;
        const long long n = (long long)cnt * tsize;
        refs_reset_kernel<<<(unsigned)((n + bs - 1) / bs), bs, 0, ctx->stream>>>(tkeys, tvals, n);
        LAUNCH_CHECK(ctx, "refs_reset_kernel");
        const dim3 grid((L + bs - 1) / bs, cnt);
        refs_insert_kernel<<<grid, bs, 0, ctx->stream>>>(d_lv + off[l], ds->d_masks, ds->d_tree, d_refs, L, tkeys,
                                                         tvals, tsize);
        LAUNCH_CHECK(ctx, "refs_insert_kernel");
        refs_lookup_kernel<<<grid, bs, 0, ctx->stream>>>(d_lv + off[l], ds->d_masks, ds->d_tree, d_refs, L, nn,
                                                         tkeys, tvals, tsize, d_out_julia);
        LAUNCH_CHECK(ctx, "refs_lookup_kernel");
    }
    return MESSI_OK;
}

size_t subcolumnrefs_work_bytes(const messi_dataset* ds)
{
    int tsize = 16;
    while (tsize < 2 * ds->L + 2) tsize <<= 1;
    std::vector<size_t> cnt(ds->H + 1, 0);
    for (int v = 0; v < ds->numnodes; v++) cnt[ds->children[2 * v] < 0 ? 0 : ds->level[v]]++;
    size_t maxw = 1;
    for (size_t c : cnt) maxw = std::max(maxw, c);
    return maxw * tsize * (sizeof(unsigned long long) + sizeof(int)) + (size_t)ds->numnodes * sizeof(int);
}

}  // namespace messi
