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

// ---------------------------------------------------------------------------
// The octree in one pass over the sorted keys.
//
// A cell of level L >= 1 is a maximal run of particles of one run whose keys share their first L
// octal digits, and it exists exactly when the range of level L - 1 around it (its parent) holds
// more than n_leaf particles (L <= KEY_LEVELS); level 0 holds one root per run.  Sizes shrink
// with the level, so for particle i, with l_i the deepest level whose range around i holds more
// than n_leaf particles, i starts a cell at every level L with d_i < L <= min(l_i + 1, KEY_LEVELS),
// d_i being the number of leading digits i shares with i - 1 (-1 at a run start, where the root
// starts too).  l_i is the largest common-digit count over the windows [j, j + n_leaf] of the run
// that contain i.  Cells are numbered level by level and, inside a level, by start -- the order
// of a level-by-level split in octant order -- so the tree is the same, cell for cell.

constexpr int OT_B = 256;      // particles per block of the one-pass build
constexpr int OT_HALO = 16;    // keys staged beyond each side of a block (windows of n_leaf <= 16 stay in it)

// the leading octal digits (levels 1..KEY_LEVELS of a 63-bit key) two keys share
__device__ __forceinline__ int key_common(uint64_t a, uint64_t b) {
    const uint64_t x = a ^ b;
    return x ? min(KEY_LEVELS, (__clzll((long long)x) - 1) / 3) : KEY_LEVELS;
}

// per particle: the levels at which it starts a cell (lo | hi << 8, empty when hi < lo), and per
// block and level the number of cells starting in the block (cnt[L * n_blocks + block])
__global__ void __launch_bounds__(OT_B) k_cell_levels(int n, int n_leaf, const uint64_t *__restrict__ keys,
                                                      const int *__restrict__ prun, const int4 *__restrict__ info,
                                                      int *__restrict__ lev, int *__restrict__ cnt) {
    __shared__ uint64_t sk[OT_B + 2 * OT_HALO];
    __shared__ int sc[MAX_LEVELS];
    const int t = threadIdx.x, b0 = blockIdx.x * OT_B, i = b0 + t;
    for (int k = t; k < OT_B + 2 * OT_HALO; k += OT_B) {
        const int g = b0 - OT_HALO + k;
        sk[k] = (g >= 0 && g < n) ? keys[g] : 0ull;
    }
    if (t < MAX_LEVELS) sc[t] = 0;
    __syncthreads();
    auto key_at = [&](int g) { const int k = g - b0 + OT_HALO; return (k >= 0 && k < OT_B + 2 * OT_HALO) ? sk[k] : keys[g]; };
    int lo = 1, hi = 0;
    if (i < n) {
        const int4 ri = info[prun[i]];
        const int rs = ri.x, re = ri.x + ri.y;
        const uint64_t ki = key_at(i);
        const int d = i == rs ? -1 : key_common(key_at(i - 1), ki);
        int ell = -1;
        const int j1 = min(i, re - 1 - n_leaf);
        for (int j = max(rs, i - n_leaf); j <= j1; ++j) ell = max(ell, key_common(key_at(j), key_at(j + n_leaf)));
        lo = d + 1;
        hi = min(ell + 1, KEY_LEVELS);
        if (i == rs) hi = max(hi, 0);
        lev[i] = lo | (hi << 8);
    }
    const int lane = t & 31;
    for (int L = 0; L < MAX_LEVELS; ++L) {
        const unsigned bal = __ballot_sync(0xffffffffu, L >= lo && L <= hi);
        if (lane == 0 && bal) atomicAdd(&sc[L], __popc(bal));
    }
    __syncthreads();
    if (t < MAX_LEVELS) cnt[(int64_t)t * gridDim.x + blockIdx.x] = sc[t];
}

// the cells: cell id = the exclusive scan of the block-and-level counts (level-major) plus the
// rank of the particle among its block's starts at that level; start, count (the end found by
// a binary search over the run's keys), level.  Also the level offsets in meta; more cells than
// the capacity sets ERR_CELL_OVERFLOW and leaves no cells.
__global__ void __launch_bounds__(OT_B) k_cell_emit(int n, int64_t cap, const uint64_t *__restrict__ keys,
                                                    const int *__restrict__ prun, const int4 *__restrict__ info,
                                                    const int *__restrict__ lev, const int *__restrict__ cnt,
                                                    const int *__restrict__ off, int *meta, int *start, int *count,
                                                    int *level) {
    __shared__ int sw[MAX_LEVELS][OT_B / 32];
    const int nb = gridDim.x, t = threadIdx.x, lane = t & 31, warp = t >> 5, i = blockIdx.x * OT_B + t;
    const int64_t last = (int64_t)(MAX_LEVELS - 1) * nb + nb - 1;
    const int64_t total = (int64_t)off[last] + cnt[last];
    const bool overflow = total > cap;
    if (blockIdx.x == 0 && t <= MAX_LEVELS) {
        meta[t] = overflow ? 0 : (t < MAX_LEVELS ? off[(int64_t)t * nb] : (int)total);
        if (t == 0 && overflow) atomicOr(&meta[META_ERR], ERR_CELL_OVERFLOW);
    }
    int lo = 1, hi = 0;
    if (i < n) {
        const int v = lev[i];
        lo = v & 255;
        hi = v >> 8;
    }
    unsigned bals[MAX_LEVELS];
#pragma unroll
    for (int L = 0; L < MAX_LEVELS; ++L) {
        bals[L] = __ballot_sync(0xffffffffu, L >= lo && L <= hi);
        if (lane == 0) sw[L][warp] = __popc(bals[L]);
    }
    __syncthreads();
    if (overflow || i >= n || hi < lo) return;
    const int4 ri = info[prun[i]];
    const int re = ri.x + ri.y;
    const uint64_t ki = keys[i];
    const unsigned below = (1u << lane) - 1u;
    for (int L = lo; L <= hi; ++L) {
        int r = __popc(bals[L] & below);
        for (int w = 0; w < warp; ++w) r += sw[L][w];
        const int id = off[(int64_t)L * nb + blockIdx.x] + r;
        // the range's end: the first particle of the run past i whose key differs in the first L digits
        int a = i + 1, b = re;
        while (a < b) {
            const int mid = (a + b) >> 1;
            if (key_common(keys[mid], ki) >= L) a = mid + 1;
            else b = mid;
        }
        start[id] = i;
        count[id] = a - i;
        level[id] = L;
    }
}

// parent, first child and child count of every cell, by binary searches over the starts of the
// levels above and below (each level's cells are sorted by start)
__global__ void k_cell_link(const int *meta, const int *start, const int *count, const int *level, int *parent,
                            int *first_child, int *n_child) {
    const int nc = meta[MAX_LEVELS];
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        const int L = level[c], s = start[c], e = s + count[c];
        int p = -1;
        if (L > 0) {   // the last cell of level L - 1 starting at or before s
            int a = meta[L - 1], b = meta[L];
            while (a < b) {
                const int mid = (a + b) >> 1;
                if (start[mid] <= s) a = mid + 1;
                else b = mid;
            }
            p = a - 1;
        }
        int f = -1, nch = 0;
        if (L < KEY_LEVELS) {   // the cells of level L + 1 starting in [s, e)
            const int a0 = meta[L + 1], b0 = meta[L + 2];
            int a = a0, b = b0;
            while (a < b) {
                const int mid = (a + b) >> 1;
                if (start[mid] < s) a = mid + 1;
                else b = mid;
            }
            const int fl = a;
            b = b0;
            while (a < b) {
                const int mid = (a + b) >> 1;
                if (start[mid] < e) a = mid + 1;
                else b = mid;
            }
            nch = a - fl;
            f = nch ? fl : -1;
        }
        parent[c] = p;
        first_child[c] = f;
        n_child[c] = nch;
    }
}

__device__ __forceinline__ double4 ldcg_d4(const double4 *p) {
    const double2 *q = reinterpret_cast<const double2 *>(p);
    const double2 a = __ldcg(q), b = __ldcg(q + 1);
    return make_double4(a.x, a.y, b.x, b.y);
}

// Moments, boxes and hmax of every cell in one launch, bottom-up.  A thread takes a leaf, then
// climbs: after its cell is written it counts itself in at the parent (arrive[], zeroed before the
// launch), and the child that arrives last sums the parent's children in octant order and climbs
// on.  The sums and their order are those of a level-by-level pass (leaf particles ascending, then
// children in octant order, one rounding per operation), independent of which thread arrives last;
// no thread waits for another (a climb ends at the first parent with children still to come, or
// at the root, after at most KEY_LEVELS steps).  Children written by other threads are read
// through L2 after the fence that orders them before their arrival.
__global__ void k_moments_up(const int *meta, const double *x, const double *y, const double *z, const double *m,
                             const double *h, const int *start, const int *count, const int *first_child,
                             const int *n_child, const int *parent, int *arrive, double4 *mom, double4 *com,
                             float4 *blo, float4 *bhi) {
    const int nc = meta[MAX_LEVELS];
    for (int c0 = blockIdx.x * blockDim.x + threadIdx.x; c0 < nc; c0 += gridDim.x * blockDim.x) {
        if (n_child[c0] != 0) continue;
        {
            double ms = 0.0, mx = 0.0, my = 0.0, mz = 0.0;
            float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
            float hm = 0.0f;
            const int s = start[c0], e = s + count[c0];
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
            mom[c0] = make_double4(mx, my, mz, ms);
            com[c0] = make_double4(__ddiv_rn(mx, ms), __ddiv_rn(my, ms), __ddiv_rn(mz, ms), ms);
            blo[c0] = make_float4(lo[0], lo[1], lo[2], 0.0f);
            bhi[c0] = make_float4(hi[0], hi[1], hi[2], hm);
        }
        int c = c0;
        for (int up = 0; up < KEY_LEVELS + 1; ++up) {
            const int p = parent[c];
            if (p < 0) break;
            // release: this cell's moments before its arrival; acquire: every sibling's arrival (and
            // so its moments) before the reads
            asm volatile("fence.acq_rel.gpu;" ::: "memory");
            if (atomicAdd(&arrive[p], 1) != n_child[p] - 1) break;
            asm volatile("fence.acq_rel.gpu;" ::: "memory");
            double ms = 0.0, mx = 0.0, my = 0.0, mz = 0.0;
            float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
            float hm = 0.0f;
            const int f = first_child[p], nch = n_child[p];
            for (int k = 0; k < nch; ++k) {
                const double4 q = ldcg_d4(mom + f + k);
                ms = __dadd_rn(ms, q.w);
                mx = __dadd_rn(mx, q.x);
                my = __dadd_rn(my, q.y);
                mz = __dadd_rn(mz, q.z);
                const float4 a = __ldcg(blo + f + k), b = __ldcg(bhi + f + k);
                lo[0] = fminf(lo[0], a.x); lo[1] = fminf(lo[1], a.y); lo[2] = fminf(lo[2], a.z);
                hi[0] = fmaxf(hi[0], b.x); hi[1] = fmaxf(hi[1], b.y); hi[2] = fmaxf(hi[2], b.z);
                hm = fmaxf(hm, b.w);
            }
            mom[p] = make_double4(mx, my, mz, ms);
            com[p] = make_double4(__ddiv_rn(mx, ms), __ddiv_rn(my, ms), __ddiv_rn(mz, ms), ms);
            blo[p] = make_float4(lo[0], lo[1], lo[2], 0.0f);
            bhi[p] = make_float4(hi[0], hi[1], hi[2], hm);
            c = p;
        }
    }
}

__global__ void k_pack_cinfo(const int *meta, const int *first_child, const int *n_child, const int *start,
                             const int *count, int4 *cinfo) {
    const int nc = meta[MAX_LEVELS];
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x)
        cinfo[c] = make_int4(first_child[c], n_child[c], start[c], count[c]);
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

// the octree over the sorted particles in one pass (k_cell_levels, a scan, k_cell_emit,
// k_cell_link), then the moments bottom-up in one launch and the packed cell records
static int enqueue_tree(sph_ctx *ctx) {
    const int64_t cap = ctx->cap;
    const int n = (int)ctx->n;
    Tree &t = ctx->tree;
    cudaStream_t st = ctx->stream;
    const double *x = FLD(ctx->F, SPH_X, cap), *y = FLD(ctx->F, SPH_Y, cap), *z = FLD(ctx->F, SPH_Z, cap);
    const double *m = FLD(ctx->F, SPH_MASS, cap), *h = FLD(ctx->F, SPH_SMTH, cap);
    const int grid = 2 * ctx->num_sms;
    const int nb = sph_div_up(n, OT_B);
    // scratch: tmp_off the particles' cell levels, tmp_cnt the block-and-level counts, tmp_b their scan
    k_cell_levels<<<nb, OT_B, 0, st>>>(n, ctx->cfg.n_leaf, ctx->keys, ctx->runs.prun, ctx->runs.info, t.tmp_off,
                                       t.tmp_cnt); ++ctx->launches;
    SPH_TRY(sph_scan_exclusive(ctx, t.tmp_cnt, t.tmp_b, nullptr, MAX_LEVELS * nb, nullptr));
    k_cell_emit<<<nb, OT_B, 0, st>>>(n, t.cap, ctx->keys, ctx->runs.prun, ctx->runs.info, t.tmp_off, t.tmp_cnt,
                                     t.tmp_b, t.meta, t.start, t.count, t.level); ++ctx->launches;
    k_cell_link<<<grid, 256, 0, st>>>(t.meta, t.start, t.count, t.level, t.parent, t.first_child, t.n_child);
    ++ctx->launches;
    // moments bottom-up in one launch (tmp_cnt, free again, counts the arrivals)
    SPH_CUDA(ctx, cudaMemsetAsync(t.tmp_cnt, 0, sizeof(int) * t.cap, st));
    // one thread per cell: the leaves' fences and arrivals all in flight at once
    const int grid_up = (int)std::min<int64_t>((t.cap + 127) / 128, 1 << 16);
    k_moments_up<<<grid_up, 128, 0, st>>>(t.meta, x, y, z, m, h, t.start, t.count, t.first_child, t.n_child,
                                          t.parent, t.tmp_cnt, t.mom, t.com, t.blo, t.bhi); ++ctx->launches;
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
    return enqueue_tree(ctx);
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
        (uintptr_t)ctx->cfg.n_leaf};
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
    t.n_cell_host = hs[MAX_LEVELS];
    int depth = 0;
    for (int l = 0; l < MAX_LEVELS; ++l)
        if (hs[l + 1] > hs[l]) depth = l;
    t.depth = depth;
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
