// Morton keys, radix sort, particle permutation and octree construction.
//
// Replaces the tree construction FDPS performs inside every
// calcForceAllAndWriteBack call (main.cpp:93-101, 139-146; tree parameters
// main.cpp:86-90).  FDPS itself is not vendored with the reference, so the
// rules below are this project's specification, restated bit-for-bit by the
// CPU oracle (oracle/sph_oracle.c: or_root_box, or_morton_keys, or_sort_perm,
// or_tree_build):
//   * root cube: centre of the particle bounding box, side = largest extent
//     x (1 + 2^-10); keys = 3 x 21-bit Morton interleave (x high, z low);
//   * stable ascending sort of the keys (ties keep the previous order);
//   * a cell is split while it holds more than n_leaf particles and is above
//     level 21; children are the non-empty octants in octant order;
//   * monopole moments are sums over the particles of a leaf (ascending) and
//     over the children of a cell (octant order), each operation rounded once
//     (no fused multiply-add), so that centres of mass and hence the gravity
//     opening decisions are bit-identical to the oracle's.
#include <algorithm>

#include "sph_internal.cuh"

namespace sph {

constexpr int SCAN_BLOCKS = 256;
constexpr int SCAN_THREADS = 256;

__device__ __forceinline__ int warp_incl_scan(int v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// inclusive block scan for blockDim.x <= 1024; returns inclusive value, *total = block sum
__device__ int block_incl_scan(int v, int *total) {
    __shared__ int ws[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    int x = warp_incl_scan(v);
    if (lane == 31) ws[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int y = (lane < nw) ? ws[lane] : 0;
        y = warp_incl_scan(y);
        if (lane < nw) ws[lane] = y;
    }
    __syncthreads();
    if (wid > 0) x += ws[wid - 1];
    *total = ws[nw - 1];
    __syncthreads();
    return x;
}

__global__ void k_scan_reduce(const int *in, LenArg len, int *part) {
    const int n = len.get();
    const int chunk = (n + gridDim.x - 1) / gridDim.x;
    const int b0 = blockIdx.x * chunk;
    const int b1 = min(n, b0 + chunk);
    int s = 0;
    for (int i = b0 + threadIdx.x; i < b1; i += blockDim.x) s += in[i];
    int tot;
    block_incl_scan(s, &tot);
    if (threadIdx.x == 0) part[blockIdx.x] = tot;
}

__global__ void k_scan_part(int *part, int nb, int *total) {
    const int t = threadIdx.x;
    const int v = (t < nb) ? part[t] : 0;
    int tot;
    const int x = block_incl_scan(v, &tot);
    if (t < nb) part[t] = x - v;
    if (t == 0 && total) *total = tot;
}

__global__ void k_scan_down(const int *in, int *out, LenArg len, const int *part) {
    const int n = len.get();
    const int chunk = (n + gridDim.x - 1) / gridDim.x;
    const int b0 = blockIdx.x * chunk;
    const int b1 = min(n, b0 + chunk);
    int base = part[blockIdx.x];
    for (int t0 = b0; t0 < b1; t0 += blockDim.x) {
        const int i = t0 + threadIdx.x;
        const int v = (i < b1) ? in[i] : 0;
        int tot;
        const int x = block_incl_scan(v, &tot);
        if (i < b1) out[i] = base + x - v;
        base += tot;
    }
}

}  // namespace sph

using namespace sph;

// exclusive scan of int32; length from device (len_dev, if non-null) or host
int sph_scan_exclusive(sph_ctx *ctx, const int *in, int *out, const int *len_dev, int len_host, int *total_dev) {
    LenArg L{len_dev, len_host, 0};
    k_scan_reduce<<<SCAN_BLOCKS, SCAN_THREADS, 0, ctx->stream>>>(in, L, ctx->scan.part); ++ctx->launches;
    k_scan_part<<<1, SCAN_BLOCKS, 0, ctx->stream>>>(ctx->scan.part, SCAN_BLOCKS, total_dev); ++ctx->launches;
    k_scan_down<<<SCAN_BLOCKS, SCAN_THREADS, 0, ctx->stream>>>(in, out, L, ctx->scan.part); ++ctx->launches;
    SPH_CUDA(ctx, cudaGetLastError());
    return SPH_OK;
}

static int scan_exclusive_diff(sph_ctx *ctx, const int *in, int *out, const int *pair_dev, int *total_dev) {
    LenArg L{pair_dev, 0, 1};
    k_scan_reduce<<<SCAN_BLOCKS, SCAN_THREADS, 0, ctx->stream>>>(in, L, ctx->scan.part); ++ctx->launches;
    k_scan_part<<<1, SCAN_BLOCKS, 0, ctx->stream>>>(ctx->scan.part, SCAN_BLOCKS, total_dev); ++ctx->launches;
    k_scan_down<<<SCAN_BLOCKS, SCAN_THREADS, 0, ctx->stream>>>(in, out, L, ctx->scan.part); ++ctx->launches;
    SPH_CUDA(ctx, cudaGetLastError());
    return SPH_OK;
}

namespace sph {

// ---------------------------------------------------------------------------
// root box and keys

constexpr int BOX_BLOCKS = 304;

__global__ void k_bbox_partial(const double *x, const double *y, const double *z, int n, double *part) {
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double p[3] = {x[i], y[i], z[i]};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            lo[d] = fmin(lo[d], p[d]);
            hi[d] = fmax(hi[d], p[d]);
        }
    }
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[d] = fmin(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
            hi[d] = fmax(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
        }
    }
    __shared__ double s[32][6];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
        for (int d = 0; d < 3; ++d) { s[wid][d] = lo[d]; s[wid][3 + d] = hi[d]; }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
            for (int d = 0; d < 3; ++d) {
                lo[d] = fmin(lo[d], s[w][d]);
                hi[d] = fmax(hi[d], s[w][3 + d]);
            }
        for (int d = 0; d < 3; ++d) { part[blockIdx.x * 6 + d] = lo[d]; part[blockIdx.x * 6 + 3 + d] = hi[d]; }
    }
}

// the root cube from the particle box exactly as or_root_box, and the opening-radius table
__device__ void root_cube(const double lo[3], const double hi[3], double theta, double *rb) {
    double L = 0.0;
    for (int d = 0; d < 3; ++d) {
        const double e = __dsub_rn(hi[d], lo[d]);
        if (e > L) L = e;
    }
    if (!(L > 0.0)) L = 1.0;
    const double half = __dmul_rn(L, 0.50048828125);
    for (int d = 0; d < 3; ++d) rb[d] = __dsub_rn(__dmul_rn(__dadd_rn(lo[d], hi[d]), 0.5), half);
    const double len = __dadd_rn(half, half);
    rb[3] = len;
    rb[4] = __ddiv_rn(2097152.0, len);
    // rc2[l] = (len / 2^l)^2 / theta^2, as or_rcrit_table
    double r = __ddiv_rn(__dmul_rn(len, len), __dmul_rn(theta, theta));
    for (int l = 0; l < MAX_LEVELS; ++l) {
        rb[8 + l] = r;
        r = __dmul_rn(r, 0.25);
    }
}

// one block reduces the partial boxes (min / max are exact in any order), then
// one thread forms the root cube
__global__ void k_bbox_final(const double *part, int nb, double theta, double *rb) {
    __shared__ double s[6][32];
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int b = threadIdx.x; b < nb; b += blockDim.x)
        for (int d = 0; d < 3; ++d) {
            lo[d] = fmin(lo[d], part[b * 6 + d]);
            hi[d] = fmax(hi[d], part[b * 6 + 3 + d]);
        }
    for (int d = 0; d < 3; ++d)
        for (int o = 16; o > 0; o >>= 1) {
            lo[d] = fmin(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
            hi[d] = fmax(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
        }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
        for (int d = 0; d < 3; ++d) {
            s[d][wid] = lo[d];
            s[3 + d][wid] = hi[d];
        }
    __syncthreads();
    if (threadIdx.x != 0) return;
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
        for (int d = 0; d < 3; ++d) {
            lo[d] = fmin(lo[d], s[d][w]);
            hi[d] = fmax(hi[d], s[3 + d][w]);
        }
    root_cube(lo, hi, theta, rb);
}

// per run: one block per tile reduces its particles' box, one block per run the tiles of the run
__device__ void block_box(double lo[3], double hi[3]) {
    __shared__ double s[6][32];
    for (int d = 0; d < 3; ++d)
        for (int o = 16; o > 0; o >>= 1) {
            lo[d] = fmin(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
            hi[d] = fmax(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
        }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0)
        for (int d = 0; d < 3; ++d) {
            s[d][wid] = lo[d];
            s[3 + d][wid] = hi[d];
        }
    __syncthreads();
    if (threadIdx.x == 0)
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w)
            for (int d = 0; d < 3; ++d) {
                lo[d] = fmin(lo[d], s[d][w]);
                hi[d] = fmax(hi[d], s[3 + d][w]);
            }
}

__global__ void k_bbox_tiles(const double *x, const double *y, const double *z, const int4 *tiles, double *part) {
    const int4 t = tiles[blockIdx.x];
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = t.x + threadIdx.x; i < t.x + t.y; i += blockDim.x) {
        const double p[3] = {x[i], y[i], z[i]};
        for (int d = 0; d < 3; ++d) {
            lo[d] = fmin(lo[d], p[d]);
            hi[d] = fmax(hi[d], p[d]);
        }
    }
    block_box(lo, hi);
    if (threadIdx.x == 0)
        for (int d = 0; d < 3; ++d) {
            part[blockIdx.x * 8 + d] = lo[d];
            part[blockIdx.x * 8 + 3 + d] = hi[d];
        }
}

__global__ void k_bbox_runs(const double *part, const int4 *info, double theta, double *rb) {
    const int4 r = info[blockIdx.x];
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int b = r.z + threadIdx.x; b < r.z + r.w; b += blockDim.x)
        for (int d = 0; d < 3; ++d) {
            lo[d] = fmin(lo[d], part[b * 8 + d]);
            hi[d] = fmax(hi[d], part[b * 8 + 3 + d]);
        }
    block_box(lo, hi);
    if (threadIdx.x == 0) root_cube(lo, hi, theta, rb + (int64_t)blockIdx.x * RB_STRIDE);
}

__device__ __forceinline__ uint64_t spread3(uint64_t v) {
    v &= 0x1fffffULL;
    v = (v | (v << 32)) & 0x1f00000000ffffULL;
    v = (v | (v << 16)) & 0x1f0000ff0000ffULL;
    v = (v | (v << 8)) & 0x100f00f00f00f00fULL;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ULL;
    v = (v | (v << 2)) & 0x1249249249249249ULL;
    return v;
}

__device__ __forceinline__ uint64_t cell_coord(double v, double lo, double scale) {
    const double t = floor(__dmul_rn(__dsub_rn(v, lo), scale));
    if (!(t > 0.0)) return 0;
    if (t >= 2097151.0) return 2097151;
    return (uint64_t)t;
}

__global__ void k_keys(const double *x, const double *y, const double *z, int n, const double *rb, uint64_t *keys,
                       uint32_t *vals, int *err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double px = x[i], py = y[i], pz = z[i];
    if (!isfinite(px) || !isfinite(py) || !isfinite(pz)) atomicOr(err, ERR_NONFINITE);
    const uint64_t qx = cell_coord(px, rb[0], rb[4]);
    const uint64_t qy = cell_coord(py, rb[1], rb[4]);
    const uint64_t qz = cell_coord(pz, rb[2], rb[4]);
    keys[i] = (spread3(qx) << 2) | (spread3(qy) << 1) | spread3(qz);
    vals[i] = (uint32_t)i;
}

// keys against the particle's own run's root cube
__global__ void k_keys_runs(const double *x, const double *y, const double *z, int n, const double *rb,
                            const int *prun, uint64_t *keys, uint32_t *vals, int *err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double *q = rb + (int64_t)prun[i] * RB_STRIDE;
    const double px = x[i], py = y[i], pz = z[i];
    if (!isfinite(px) || !isfinite(py) || !isfinite(pz)) atomicOr(err, ERR_NONFINITE);
    const uint64_t qx = cell_coord(px, q[0], q[4]);
    const uint64_t qy = cell_coord(py, q[1], q[4]);
    const uint64_t qz = cell_coord(pz, q[2], q[4]);
    keys[i] = (spread3(qx) << 2) | (spread3(qy) << 1) | spread3(qz);
    vals[i] = (uint32_t)i;
}

// ---------------------------------------------------------------------------
// LSD radix sort of (key, value), 8 passes of 8 bits.  Each pass: per-tile
// digit histogram, one exclusive scan over (digit, tile), then a stable
// in-tile ranking and a scatter.  With a tile table (tiles aligned to run
// starts; each entry: start, length, histogram base, tiles of its run) the
// histogram is laid out run by run, digit-major within a run, so the one scan
// yields offsets that keep every run in its own range: a segmented sort.
// Without one, tile b covers [b * RS_TILE, ...) and the layout is digit-major.

// RS_THREADS, RS_ITEMS, RS_TILE: sph_internal.cuh

__device__ __forceinline__ int4 rs_tile(const int4 *tiles, int n, int nb) {
    if (tiles) return tiles[blockIdx.x];
    const int s = blockIdx.x * RS_TILE;
    return make_int4(s, min(RS_TILE, n - s), blockIdx.x, nb);
}

__global__ void k_rs_hist(const uint64_t *keys, int n, int shift, uint32_t *hist, int nb, const int4 *tiles) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int4 tl = rs_tile(tiles, n, nb);
#pragma unroll
    for (int k = 0; k < RS_ITEMS; ++k) {
        const int p = k * RS_THREADS + threadIdx.x;
        if (p < tl.y) atomicAdd(&h[(keys[tl.x + p] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[tl.z + threadIdx.x * tl.w] = h[threadIdx.x];
}

// Stable in-tile ranking by warp multisplit: each warp ranks its 256 keys
// (eight rounds of 32 consecutive keys) with __match_any_sync against
// per-warp digit counters; the counters of the eight warps are then turned
// into per-digit offsets, the tile is reordered by digit in shared memory and
// written out in runs of equal digit.
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_WKEYS = RS_TILE / RS_WARPS;
static_assert(RS_THREADS == 256, "one thread per digit in the offset step");

__global__ void __launch_bounds__(RS_THREADS) k_rs_scatter(const uint64_t *kin, const uint32_t *vin, uint64_t *kout,
                                                           uint32_t *vout, int n, int shift, const uint32_t *off,
                                                           int nb, const int4 *tiles) {
    __shared__ uint64_t sk[RS_TILE];
    __shared__ uint32_t sv[RS_TILE];
    __shared__ uint32_t wc[RS_WARPS][256];   // per-warp digit counts, then per-warp offsets within a digit
    __shared__ uint32_t dstart[256];         // first tile position of each digit
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const unsigned lt = (1u << lane) - 1u;
    const int4 tl = rs_tile(tiles, n, nb);
    const int base = tl.x;
    const int cnt = tl.y;
    for (int k = t; k < RS_WARPS * 256; k += RS_THREADS) (&wc[0][0])[k] = 0u;
    __syncthreads();
    uint64_t key[RS_ITEMS];
    uint32_t val[RS_ITEMS], rk[RS_ITEMS];
    int dg[RS_ITEMS];
#pragma unroll
    for (int r = 0; r < RS_ITEMS; ++r) {
        const int p = w * RS_WKEYS + r * 32 + lane;
        const bool ok = p < cnt;
        key[r] = ok ? kin[base + p] : 0ULL;
        val[r] = ok ? vin[base + p] : 0u;
        const int d = ok ? (int)((key[r] >> shift) & 255u) : 256;   // 256: no item
        dg[r] = d;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        uint32_t b0 = 0;
        if (ok) b0 = wc[w][d];
        rk[r] = b0 + (uint32_t)__popc(peers & lt);
        __syncwarp();
        if (ok && lane == __ffs(peers) - 1) wc[w][d] = b0 + (uint32_t)__popc(peers);
        __syncwarp();
    }
    __syncthreads();
    {
        uint32_t c = 0;
        for (int ww = 0; ww < RS_WARPS; ++ww) {
            const uint32_t v = wc[ww][t];
            wc[ww][t] = c;
            c += v;
        }
        int tot;
        const int incl = block_incl_scan((int)c, &tot);
        dstart[t] = (uint32_t)incl - c;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < RS_ITEMS; ++r) {
        const int d = dg[r];
        if (d < 256) {
            const uint32_t p = dstart[d] + wc[w][d] + rk[r];
            sk[p] = key[r];
            sv[p] = val[r];
        }
    }
    __syncthreads();
    for (int k = 0; k < RS_ITEMS; ++k) {
        const int p = k * RS_THREADS + t;
        if (p < cnt) {
            const uint64_t kk = sk[p];
            const int d = (int)((kk >> shift) & 255u);
            const uint32_t g = off[tl.z + d * tl.w] + (uint32_t)p - dstart[d];
            kout[g] = kk;
            vout[g] = sv[p];
        }
    }
}

__global__ void k_u32_to_i32_copy(const uint32_t *a, int *b, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (int)a[i];
}

// gather all particle arrays through the permutation
__global__ void k_permute(const double *F, double *F2, int64_t cap, int n, const uint32_t *perm, const int64_t *id,
                          int64_t *id2, const int32_t *slot, int32_t *slot2, const int32_t *mat, int32_t *mat2,
                          const int *prun, int *prun2) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int src = (int)perm[k];
#pragma unroll 4
    for (int f = 0; f < SPH_NFIELD; ++f) F2[(int64_t)f * cap + k] = F[(int64_t)f * cap + src];
    id2[k] = id[src];
    slot2[k] = slot[src];
    mat2[k] = mat[src];
    prun2[k] = prun[src];
}

// ---------------------------------------------------------------------------
// octree

// level 0: one root per run (cell r = run r)
__global__ void k_tree_init(int R, const int4 *info, int *meta, int *start, int *count, int *level, int *parent,
                            int *first_child, int *n_child) {
    for (int r = threadIdx.x; r < R; r += blockDim.x) {
        const int4 q = info[r];
        start[r] = q.x;
        count[r] = q.y;
        level[r] = 0;
        parent[r] = -1;
        first_child[r] = -1;
        n_child[r] = 0;
    }
    if (threadIdx.x == 0) {
        for (int k = 0; k < META_N; ++k) meta[k] = 0;
        meta[0] = 0;
        meta[1] = R;
    }
}

__device__ __forceinline__ int digit_at(uint64_t key, int level) {
    return (int)((key >> (3 * (KEY_LEVELS - level))) & 7ULL);
}

// Children of the cells of level l: the first position of each octant
// (digit l + 1) in the cell's sorted key range.  Cells of up to SPLIT_SMALL
// particles are searched by one thread each (binary searches over a range
// that sits in L1); larger cells, the top of the tree, by a warp each with
// 32-way searches, so level 0 over all n particles takes a few dependent
// loads per octant instead of log2 n.
constexpr int SPLIT_SMALL = 256;

__device__ __forceinline__ void split_store(int *tb, int s, int e, const int *bnd, int *nch) {
    int prev = s, k = 0;
    tb[0] = s;
    for (int oct = 1; oct < 8; ++oct) {
        tb[oct] = bnd[oct];
        k += (bnd[oct] > prev);
        prev = bnd[oct];
    }
    tb[8] = e;
    *nch = k + (e > prev);
}

// first position in [a, e) whose digit at `lev` is >= oct (keys ascending within the range)
__device__ __forceinline__ int split_search1(const uint64_t *keys, int lev, int a, int e, int oct) {
    int len = e - a;
    while (len > 0) {
        const int half = len >> 1;
        if (digit_at(keys[a + half], lev) < oct) {
            a += half + 1;
            len -= half + 1;
        } else {
            len = half;
        }
    }
    return a;
}

// K independent searches of split_search1 interleaved, so their loads overlap: search q looks
// in [a[q], e[q]) for digit o[q] and leaves the answer in a[q]
template <int K>
__device__ __forceinline__ void split_searchK(const uint64_t *keys, int lev, int (&a)[K], const int (&e)[K],
                                              const int (&o)[K]) {
    int len[K];
#pragma unroll
    for (int q = 0; q < K; ++q) len[q] = e[q] - a[q];
    for (;;) {
        bool any = false;
        bool lt[K];
#pragma unroll
        for (int q = 0; q < K; ++q) {
            lt[q] = len[q] > 0 && digit_at(keys[a[q] + (len[q] >> 1)], lev) < o[q];
            any = any || len[q] > 0;
        }
        if (!any) break;
#pragma unroll
        for (int q = 0; q < K; ++q) {
            if (len[q] <= 0) continue;
            const int h = len[q] >> 1;
            if (lt[q]) {
                a[q] += h + 1;
                len[q] -= h + 1;
            } else {
                len[q] = h;
            }
        }
    }
}


// the octant boundaries of one big cell [s, e) by a whole warp, 32-way searches
__device__ __forceinline__ void split_big(const uint64_t *keys, int l, int lane, int c, int L0, int s, int e,
                                          int *tmp_cnt, int *tmp_b) {
    int bnd[8];
    int lo = s;
    for (int oct = 1; oct < 8; ++oct) {
        // first position in [lo, e) with digit >= oct; the answer lies in [a, b]
        int a = lo, b = e;
        while (b - a > 32) {
            const int step = (b - a + 31) >> 5;
            const int p = a + lane * step;
            const bool below = p < b && digit_at(keys[p], l + 1) < oct;
            const int kb = __popc(__ballot_sync(0xffffffffu, below));
            if (kb == 0) {
                b = a;
            } else {
                const int na = a + (kb - 1) * step + 1;
                b = min(b, a + kb * step);
                a = na;
            }
        }
        if (b > a) {
            const int p = a + lane;
            const bool below = p < b && digit_at(keys[p], l + 1) < oct;
            a += __popc(__ballot_sync(0xffffffffu, below));
        }
        bnd[oct] = a;
        lo = a;
    }
    if (lane == 0) {
        int nch = 0;
        split_store(tmp_b + (int64_t)(c - L0) * 9, s, e, bnd, &nch);
        tmp_cnt[c - L0] = nch;
    }
}

// Small cells (<= SPLIT_SMALL particles) go to one thread each, big ones to one warp each,
// spread over all warps of the grid: a level with fewer cells than warps gives every cell its
// own warp (the top levels hold a few hundred big cells), a larger one is scanned 32 cells at
// a time per warp.
__global__ void __launch_bounds__(256) k_split(int l, int n_leaf, const uint64_t *keys, const int *meta,
                                               const int *start, const int *count, int *tmp_cnt, int *tmp_b) {
    const int L0 = meta[l], L1 = meta[l + 1], nL = L1 - L0;
    const int gt = blockIdx.x * blockDim.x + threadIdx.x, nt = gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31, gw = gt >> 5, nw = nt >> 5;
    const bool deep = l < KEY_LEVELS;
    for (int c = L0 + gt; c < L1; c += nt) {
        const int s = start[c], cnt = count[c];
        if (cnt > SPLIT_SMALL && deep) continue;   // a warp's
        int nch = 0;
        if (cnt > n_leaf && deep) {
            // the seven octant boundaries in three rounds of independent searches (octant 4;
            // then 2 and 6; then 1, 3, 5, 7), each search over the range its neighbours bound
            int bnd[8];
            const int e = s + cnt;
            bnd[4] = split_search1(keys, l + 1, s, e, 4);
            {
                int a2[2] = {s, bnd[4]};
                split_searchK<2>(keys, l + 1, a2, {bnd[4], e}, {2, 6});
                bnd[2] = a2[0];
                bnd[6] = a2[1];
            }
            {
                int a4[4] = {s, bnd[2], bnd[4], bnd[6]};
                split_searchK<4>(keys, l + 1, a4, {bnd[2], bnd[4], bnd[6], e}, {1, 3, 5, 7});
                bnd[1] = a4[0];
                bnd[3] = a4[1];
                bnd[5] = a4[2];
                bnd[7] = a4[3];
            }
            split_store(tmp_b + (int64_t)(c - L0) * 9, s, e, bnd, &nch);
        }
        tmp_cnt[c - L0] = nch;
    }
    if (!deep) return;
    if (nL <= nw) {
        if (gw < nL) {
            const int c = L0 + gw;
            const int s = start[c], cnt = count[c];
            if (cnt > SPLIT_SMALL) split_big(keys, l, lane, c, L0, s, s + cnt, tmp_cnt, tmp_b);
        }
        return;
    }
    for (int q0 = gw * 32; q0 < nL; q0 += nw * 32) {
        const int q = q0 + lane;
        const int cl = q < nL ? count[L0 + q] : 0;
        unsigned big = __ballot_sync(0xffffffffu, cl > SPLIT_SMALL);
        while (big) {
            const int k = __ffs(big) - 1;
            big &= big - 1;
            const int c = L0 + q0 + k;
            const int s = start[c];
            split_big(keys, l, lane, c, L0, s, s + __shfl_sync(0xffffffffu, cl, k), tmp_cnt, tmp_b);
        }
    }
}

__global__ void k_emit(int l, int64_t cap, int *meta, const int *tmp_cnt, const int *tmp_off, const int *tmp_b,
                       const int *total, int *start, int *count, int *level, int *parent, int *first_child,
                       int *n_child) {
    const int L0 = meta[l], L1 = meta[l + 1];
    const int tot = *total;
    const bool overflow = (int64_t)L1 + tot > cap;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        meta[l + 2] = overflow ? L1 : L1 + tot;
        if (overflow) atomicOr(&meta[META_ERR], ERR_CELL_OVERFLOW);
    }
    for (int c = L0 + blockIdx.x * blockDim.x + threadIdx.x; c < L1; c += gridDim.x * blockDim.x) {
        const int nch = overflow ? 0 : tmp_cnt[c - L0];
        n_child[c] = nch;
        if (nch == 0) {
            first_child[c] = -1;
            continue;
        }
        const int first = L1 + tmp_off[c - L0];
        first_child[c] = first;
        const int *b = tmp_b + (int64_t)(c - L0) * 9;
        int k = 0;
        for (int oct = 0; oct < 8; ++oct) {
            const int a = b[oct], e = b[oct + 1];
            if (e <= a) continue;
            const int ch = first + k++;
            start[ch] = a;
            count[ch] = e - a;
            level[ch] = l + 1;
            parent[ch] = c;
            first_child[ch] = -1;
            n_child[ch] = 0;
        }
    }
}

// moments, bounding boxes and hmax of one level (children first)
__global__ void k_moments(int l, const int *meta, const double *x, const double *y, const double *z, const double *m,
                          const double *h, const int *start, const int *count, const int *first_child,
                          const int *n_child, double4 *mom, double4 *com, float4 *blo, float4 *bhi) {
    const int L0 = meta[l], L1 = meta[l + 1];
    for (int c = L0 + blockIdx.x * blockDim.x + threadIdx.x; c < L1; c += gridDim.x * blockDim.x) {
        double ms = 0.0, mx = 0.0, my = 0.0, mz = 0.0;
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        float hm = 0.0f;
        const int nch = n_child[c];
        if (nch == 0) {
            // the box and hmax in FP32: rounding down (up) is monotone, so the min (max) of the
            // rounded values is the rounded min (max), without FP64 comparisons
            const int s = start[c], e = s + count[c];
            for (int j = s; j < e; ++j) {
                const double mj = m[j], xj = x[j], yj = y[j], zj = z[j];
                ms = __dadd_rn(ms, mj);
                mx = __dadd_rn(mx, __dmul_rn(mj, xj));
                my = __dadd_rn(my, __dmul_rn(mj, yj));
                mz = __dadd_rn(mz, __dmul_rn(mj, zj));
                lo[0] = fminf(lo[0], __double2float_rd(xj)); hi[0] = fmaxf(hi[0], __double2float_ru(xj));
                lo[1] = fminf(lo[1], __double2float_rd(yj)); hi[1] = fmaxf(hi[1], __double2float_ru(yj));
                lo[2] = fminf(lo[2], __double2float_rd(zj)); hi[2] = fmaxf(hi[2], __double2float_ru(zj));
                hm = fmaxf(hm, __double2float_ru(h[j]));
            }
        } else {
            const int f = first_child[c];
            for (int k = 0; k < nch; ++k) {
                const double4 q = mom[f + k];
                ms = __dadd_rn(ms, q.w);
                mx = __dadd_rn(mx, q.x);
                my = __dadd_rn(my, q.y);
                mz = __dadd_rn(mz, q.z);
                const float4 a = blo[f + k], b = bhi[f + k];
                lo[0] = fminf(lo[0], a.x); lo[1] = fminf(lo[1], a.y); lo[2] = fminf(lo[2], a.z);
                hi[0] = fmaxf(hi[0], b.x); hi[1] = fmaxf(hi[1], b.y); hi[2] = fmaxf(hi[2], b.z);
                hm = fmaxf(hm, b.w);
            }
        }
        mom[c] = make_double4(mx, my, mz, ms);
        com[c] = make_double4(__ddiv_rn(mx, ms), __ddiv_rn(my, ms), __ddiv_rn(mz, ms), ms);
        blo[c] = make_float4(lo[0], lo[1], lo[2], 0.0f);
        bhi[c] = make_float4(hi[0], hi[1], hi[2], hm);
    }
}

__global__ void k_pack_cinfo(const int *meta, const int *first_child, const int *n_child, const int *start,
                             const int *count, int4 *cinfo) {
    const int nc = meta[MAX_LEVELS];
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x)
        cinfo[c] = make_int4(first_child[c], n_child[c], start[c], count[c]);
}

// after the levels [0, Lb) were split: flags a cell of level Lb that would still split (the tree
// is deeper than this build went) and marks the levels below Lb empty
__global__ void k_tree_tail(int Lb, int n_leaf, int *meta, const int *count) {
    const int L0 = meta[Lb], L1 = meta[Lb + 1];
    if (Lb < KEY_LEVELS)
        for (int c = L0 + blockIdx.x * blockDim.x + threadIdx.x; c < L1; c += gridDim.x * blockDim.x)
            if (count[c] > n_leaf) atomicOr(&meta[META_ERR], ERR_TREE_DEEPER);
    if (blockIdx.x == 0)
        for (int l = Lb + 2 + threadIdx.x; l <= MAX_LEVELS; l += blockDim.x) meta[l] = L1;
}

__global__ void k_hmax(int l, const int *meta, const double *h, const int *start, const int *count,
                       const int *first_child, const int *n_child, float4 *bhi) {
    const int L0 = meta[l], L1 = meta[l + 1];
    for (int c = L0 + blockIdx.x * blockDim.x + threadIdx.x; c < L1; c += gridDim.x * blockDim.x) {
        float hm = 0.0f;
        const int nch = n_child[c];
        if (nch == 0) {
            for (int j = start[c]; j < start[c] + count[c]; ++j) hm = fmaxf(hm, __double2float_ru(h[j]));
        } else {
            for (int k = 0; k < nch; ++k) hm = fmaxf(hm, bhi[first_child[c] + k].w);
        }
        bhi[c].w = hm;
    }
}

}  // namespace sph

// ---------------------------------------------------------------------------
// host side

template <class T>
static int dalloc(sph_ctx *ctx, T **p, int64_t n) {
    if (*p) cudaFree(*p);
    *p = nullptr;
    if (n <= 0) n = 1;
    cudaError_t e = cudaMalloc((void **)p, sizeof(T) * (size_t)n);
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return sph_fail(ctx, SPH_ERR_OOM, "device allocation of %lld bytes failed: %s",
                        (long long)(sizeof(T) * (size_t)n), cudaGetErrorString(e));
    }
    return SPH_OK;
}

int sph_tree_reserve(sph_ctx *ctx, int64_t n) {
    Tree &t = ctx->tree;
    const int64_t want = 2 * n + 64;
    if (t.cap < want) {
        const int64_t c = want + want / 4;
        SPH_TRY(dalloc(ctx, &t.start, c));
        SPH_TRY(dalloc(ctx, &t.count, c));
        SPH_TRY(dalloc(ctx, &t.level, c));
        SPH_TRY(dalloc(ctx, &t.first_child, c));
        SPH_TRY(dalloc(ctx, &t.n_child, c));
        SPH_TRY(dalloc(ctx, &t.parent, c));
        SPH_TRY(dalloc(ctx, &t.mom, c));
        SPH_TRY(dalloc(ctx, &t.com, c));
        SPH_TRY(dalloc(ctx, &t.blo, c));
        SPH_TRY(dalloc(ctx, &t.bhi, c));
        SPH_TRY(dalloc(ctx, &t.tmp_cnt, c));
        SPH_TRY(dalloc(ctx, &t.tmp_off, c));
        SPH_TRY(dalloc(ctx, &t.tmp_b, 9 * c));
        SPH_TRY(dalloc(ctx, &t.cinfo, c));
        SPH_TRY(dalloc(ctx, &ctx->grav.is_group, c));
        t.cap = c;
    }
    if (!t.meta) SPH_TRY(dalloc(ctx, &t.meta, META_N));
    if (t.rb_cap < ctx->runs.cap_R) {
        SPH_TRY(dalloc(ctx, &t.rb, (int64_t)RB_STRIDE * ctx->runs.cap_R));
        t.rb_cap = ctx->runs.cap_R;
    }
    Sort &s = ctx->sort;
    if (s.cap < n) {
        const int64_t c = n + n / 8 + 1024;
        SPH_TRY(dalloc(ctx, &s.k0, c));
        SPH_TRY(dalloc(ctx, &s.k1, c));
        SPH_TRY(dalloc(ctx, &s.v0, c));
        SPH_TRY(dalloc(ctx, &s.v1, c));
        s.cap = c;
    }
    if (s.nblocks_cap < ctx->runs.cap_T) {   // tiles of all runs (each run starts a tile)
        SPH_TRY(dalloc(ctx, &s.hist, 256 * (int64_t)ctx->runs.cap_T));
        SPH_TRY(dalloc(ctx, &s.hoff, 256 * (int64_t)ctx->runs.cap_T));
        s.nblocks_cap = ctx->runs.cap_T;
    }
    if (!ctx->scan.part) {
        SPH_TRY(dalloc(ctx, &ctx->scan.part, SCAN_BLOCKS + 1));
        SPH_TRY(dalloc(ctx, &ctx->scan.total, 16));
    }
    return SPH_OK;
}

static int radix_sort(sph_ctx *ctx, int n) {
    Sort &s = ctx->sort;
    const int nb = ctx->runs.T;
    const int4 *tiles = ctx->runs.tiles;
    static_assert(RS_TILE == RUN_TILE, "run tiles are radix tiles");
    uint64_t *ka = s.k0, *kb = s.k1;
    uint32_t *va = s.v0, *vb = s.v1;
    for (int pass = 0; pass < 8; ++pass) {
        const int shift = pass * 8;
        k_rs_hist<<<nb, RS_THREADS, 0, ctx->stream>>>(ka, n, shift, s.hist, nb, tiles); ++ctx->launches;
        SPH_TRY(sph_scan_exclusive(ctx, (const int *)s.hist, (int *)s.hoff, nullptr, 256 * nb, nullptr));
        k_rs_scatter<<<nb, RS_THREADS, 0, ctx->stream>>>(ka, va, kb, vb, n, shift, s.hoff, nb, tiles); ++ctx->launches;
        std::swap(ka, kb);
        std::swap(va, vb);
    }
    SPH_CUDA(ctx, cudaGetLastError());
    // 8 passes: the result is back in k0 / v0
    return SPH_OK;
}

// the octree over the sorted particles, level by level (level sizes stay on the device): the
// levels [0, Lb) are split, then a tail kernel checks that level Lb needs no split (else the
// host builds again with every level) and marks the deeper levels empty; moments bottom-up
static int enqueue_tree(sph_ctx *ctx, int Lb) {
    const int64_t cap = ctx->cap;
    Tree &t = ctx->tree;
    cudaStream_t st = ctx->stream;
    const double *x = FLD(ctx->F, SPH_X, cap), *y = FLD(ctx->F, SPH_Y, cap), *z = FLD(ctx->F, SPH_Z, cap);
    const double *m = FLD(ctx->F, SPH_MASS, cap), *h = FLD(ctx->F, SPH_SMTH, cap);
    const int grid = 2 * ctx->num_sms;
    for (int l = 0; l < Lb; ++l) {
        k_split<<<grid, 256, 0, st>>>(l, ctx->cfg.n_leaf, ctx->keys, t.meta, t.start, t.count, t.tmp_cnt, t.tmp_b); ++ctx->launches;
        SPH_TRY(scan_exclusive_diff(ctx, t.tmp_cnt, t.tmp_off, t.meta + l, ctx->scan.total));
        k_emit<<<grid, 256, 0, st>>>(l, t.cap, t.meta, t.tmp_cnt, t.tmp_off, t.tmp_b, ctx->scan.total, t.start,
                                     t.count, t.level, t.parent, t.first_child, t.n_child); ++ctx->launches;
    }
    k_tree_tail<<<grid, 256, 0, st>>>(Lb, ctx->cfg.n_leaf, t.meta, t.count); ++ctx->launches;
    for (int l = Lb; l >= 0; --l)
        k_moments<<<grid, 128, 0, st>>>(l, t.meta, x, y, z, m, h, t.start, t.count, t.first_child, t.n_child,
                                        t.mom, t.com, t.blo, t.bhi); ++ctx->launches;
    k_pack_cinfo<<<grid, 256, 0, st>>>(t.meta, t.first_child, t.n_child, t.start, t.count, t.cinfo);
    ++ctx->launches;
    SPH_CUDA(ctx, cudaGetLastError());
    return SPH_OK;
}

// the device work of sph_sort_and_build up to the cell-count read: root cubes, keys, the
// segmented radix sort, the permutation (and its host-side buffer swaps), the octree levels,
// the moments.  No host synchronisation and no allocation inside, so it can be captured.
static int enqueue_sort_tree(sph_ctx *ctx) {
    const int n = (int)ctx->n;
    const int64_t cap = ctx->cap;
    double *x = FLD(ctx->F, SPH_X, cap), *y = FLD(ctx->F, SPH_Y, cap), *z = FLD(ctx->F, SPH_Z, cap);
    Tree &t = ctx->tree;
    cudaStream_t st = ctx->stream;
    // root cube of every run (one block per tile, then one per run)
    const Runs &R = ctx->runs;
    k_bbox_tiles<<<R.T, 256, 0, st>>>(x, y, z, R.tiles, R.part); ++ctx->launches;
    k_bbox_runs<<<R.R, 256, 0, st>>>(R.part, R.info, ctx->cfg.theta, t.rb); ++ctx->launches;
    k_tree_init<<<1, 256, 0, st>>>(R.R, R.info, t.meta, t.start, t.count, t.level, t.parent, t.first_child,
                                   t.n_child); ++ctx->launches;
    k_keys_runs<<<sph_div_up(n, 256), 256, 0, st>>>(x, y, z, n, t.rb, R.prun, ctx->sort.k0, ctx->sort.v0,
                                                    t.meta + META_ERR); ++ctx->launches;
    SPH_TRY(radix_sort(ctx, n));
    // permute the particle state into key order
    k_permute<<<sph_div_up(n, 256), 256, 0, st>>>(ctx->F, ctx->F2, cap, n, ctx->sort.v0, ctx->id, ctx->id2,
                                                  ctx->slot, ctx->slot2, ctx->mat, ctx->mat2, R.prun,
                                                  ctx->runs.prun2); ++ctx->launches;
    std::swap(ctx->F, ctx->F2);
    std::swap(ctx->runs.prun, ctx->runs.prun2);
    std::swap(ctx->id, ctx->id2);
    std::swap(ctx->slot, ctx->slot2);
    std::swap(ctx->mat, ctx->mat2);
    SPH_CUDA(ctx, cudaMemcpyAsync(ctx->keys, ctx->sort.k0, sizeof(uint64_t) * n, cudaMemcpyDeviceToDevice, st));
    SPH_TRY(time_mark(ctx, SEG_SORT));
    return enqueue_tree(ctx, t.levels);
}

// Everything the captured work depends on: sizes and every buffer it touches.  The permutation
// swaps the state buffers, so a step alternates between two keys.
static void graph_key(const sph_ctx *ctx, uintptr_t key[GRAPH_KEY_N]) {
    const Tree &t = ctx->tree;
    const uintptr_t k[GRAPH_KEY_N] = {
        (uintptr_t)ctx->n,         (uintptr_t)ctx->cap,        (uintptr_t)ctx->runs.R,   (uintptr_t)ctx->runs.T,
        (uintptr_t)ctx->F,         (uintptr_t)ctx->F2,         (uintptr_t)ctx->id,       (uintptr_t)ctx->slot,
        (uintptr_t)ctx->mat,       (uintptr_t)ctx->runs.prun,  (uintptr_t)ctx->keys,     (uintptr_t)ctx->sort.k0,
        (uintptr_t)ctx->sort.hist, (uintptr_t)t.start,         (uintptr_t)t.rb,          (uintptr_t)t.cap,
        (uintptr_t)ctx->runs.tiles, (uintptr_t)ctx->runs.part, (uintptr_t)ctx->scan.part, (uintptr_t)t.cinfo,
        (uintptr_t)t.levels};
    for (int i = 0; i < GRAPH_KEY_N; ++i) key[i] = k[i];
}

// replays the captured sort + octree for this key (capturing it the first time)
static int sort_tree_graph(sph_ctx *ctx) {
    uintptr_t key[GRAPH_KEY_N];
    graph_key(ctx, key);
    TreeGraph *g = nullptr;
    for (TreeGraph &c : ctx->tree_graphs)
        if (c.exec && std::equal(key, key + GRAPH_KEY_N, c.key)) g = &c;
    if (g) {
        // the captured work's host side: the buffer swaps of the permutation
        std::swap(ctx->F, ctx->F2);
        std::swap(ctx->runs.prun, ctx->runs.prun2);
        std::swap(ctx->id, ctx->id2);
        std::swap(ctx->slot, ctx->slot2);
        std::swap(ctx->mat, ctx->mat2);
        ctx->launches += g->launches;
        ctx->graph_replays += 1;
    } else {
        g = &ctx->tree_graphs[ctx->graph_next];
        ctx->graph_next = (ctx->graph_next + 1) % (int)(sizeof(ctx->tree_graphs) / sizeof(ctx->tree_graphs[0]));
        if (g->exec) cudaGraphExecDestroy(g->exec);
        g->exec = nullptr;
        cudaGraph_t graph = nullptr;
        const int64_t l0 = ctx->launches;
        SPH_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        const int rc = enqueue_sort_tree(ctx);
        const cudaError_t ce = cudaStreamEndCapture(ctx->stream, &graph);
        if (rc != SPH_OK) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (ce != cudaSuccess) {
            cudaGetLastError();
            return sph_fail(ctx, SPH_ERR_CUDA, "capture of the octree build failed: %s", cudaGetErrorString(ce));
        }
        const cudaError_t ie = cudaGraphInstantiate(&g->exec, graph, 0);
        cudaGraphDestroy(graph);
        if (ie != cudaSuccess) {
            g->exec = nullptr;
            cudaGetLastError();
            return sph_fail(ctx, SPH_ERR_CUDA, "instantiation of the octree build failed: %s", cudaGetErrorString(ie));
        }
        std::copy(key, key + GRAPH_KEY_N, g->key);
        g->launches = ctx->launches - l0;
        ctx->graph_captures += 1;
    }
    SPH_CUDA(ctx, cudaGraphLaunch(g->exec, ctx->stream));
    return SPH_OK;
}

int sph_sort_and_build(sph_ctx *ctx) {
    const int n = (int)ctx->n;
    Tree &t = ctx->tree;
    SPH_TRY(sph_tree_reserve(ctx, n));
    cudaStream_t st = ctx->stream;
    // With event timing on the work is launched directly (its segments are timed); otherwise the
    // ~170 launches of the sort and the level loop replay as one CUDA graph.
    if (ctx->timing || !ctx->use_graphs) SPH_TRY(enqueue_sort_tree(ctx));
    else SPH_TRY(sort_tree_graph(ctx));
    // bring back the cell count and the error word (one small synchronous read per tree)
    int *hs = (int *)ctx->host_scalars;
    SPH_CUDA(ctx, cudaMemcpyAsync(hs, t.meta, sizeof(int) * META_N, cudaMemcpyDeviceToHost, st));
    SPH_CUDA(ctx, cudaStreamSynchronize(st));
    if (hs[META_ERR] & ERR_NONFINITE) return sph_fail(ctx, SPH_ERR_NONFINITE, "non-finite particle position");
    if (hs[META_ERR] & ERR_CELL_OVERFLOW) return sph_fail(ctx, SPH_ERR_CAPACITY, "octree cell capacity exceeded");
    if (hs[META_ERR] & ERR_TREE_DEEPER) {   // deeper than the last tree plus two levels: every level
        SPH_CUDA(ctx, cudaMemsetAsync(t.meta + META_ERR, 0, sizeof(int), st));
        t.levels = KEY_LEVELS;
        SPH_TRY(enqueue_tree(ctx, KEY_LEVELS));
        SPH_CUDA(ctx, cudaMemcpyAsync(hs, t.meta, sizeof(int) * META_N, cudaMemcpyDeviceToHost, st));
        SPH_CUDA(ctx, cudaStreamSynchronize(st));
        if (hs[META_ERR] & ERR_CELL_OVERFLOW) return sph_fail(ctx, SPH_ERR_CAPACITY, "octree cell capacity exceeded");
    }
    t.n_cell_host = hs[MAX_LEVELS];
    int depth = 0;
    for (int l = 0; l < MAX_LEVELS; ++l)
        if (hs[l + 1] > hs[l]) depth = l;
    t.depth = depth;
    t.levels = std::min(KEY_LEVELS, depth + 2);
    ctx->grav.valid = false;
    ctx->grav.counts_valid = false;
    SPH_TRY(time_mark(ctx, SEG_TREE));
    return sph_nbr_prepare(ctx);
}

int sph_tree_refresh_hmax(sph_ctx *ctx) {
    Tree &t = ctx->tree;
    const double *h = FLD(ctx->F, SPH_SMTH, ctx->cap);
    const int grid = 2 * ctx->num_sms;
    for (int l = t.depth; l >= 0; --l)
        k_hmax<<<grid, 128, 0, ctx->stream>>>(l, t.meta, h, t.start, t.count, t.first_child, t.n_child, t.bhi); ++ctx->launches;
    SPH_CUDA(ctx, cudaGetLastError());
    return SPH_OK;
}
