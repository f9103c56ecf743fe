// Gravity interaction lists on the device (the SPH neighbour lists are in
// sph_nbr.cu).
//
// Gravity (TreeForForceLong::Monopole, main.cpp:83,90): one warp per i-group
// (cells with <= n_group particles whose parent holds more) walks the tree
// with the group's FP64 bounding box; a child is opened iff
// dmin^2(box, com) <= (side / theta)^2.  Opened leaves give EPJ particle
// ranges, unopened children of opened cells give SPJ monopoles, in the
// breadth-first order of the oracle's or_grav_walk.  Counting pass, scan,
// filling pass.
#include <algorithm>

#include "sph_internal.cuh"

namespace sph {

constexpr int LIST_WARPS = 4;
constexpr int CAND_CAP = 512;
constexpr int STACK_CAP = 256;
constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ double warp_min_d(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(FULL, v, o));
    return v;
}
__device__ __forceinline__ double warp_max_d(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(FULL, v, o));
    return v;
}
__device__ __forceinline__ int warp_max_i(int v) {
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(FULL, v, o));
    return v;
}

struct TreeView {
    const int *start, *count, *first_child, *n_child, *level;
    const float4 *blo, *bhi;
    const double4 *com;
};

// --------------------------------------------------------------------------
// gravity i-groups and interaction lists

__global__ void k_mark_groups(const int *meta, const int *count, const int *parent, int n_group, int *is_group) {
    const int nc = meta[MAX_LEVELS];
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        const int p = parent[c];
        is_group[c] = (count[c] <= n_group && (p < 0 || count[p] > n_group)) ? 1 : 0;
    }
    // cells that are leaves but still above n_group (only possible at the deepest level) are groups too
}

__global__ void k_mark_groups_fix(const int *meta, const int *count, const int *parent, const int *n_child,
                                  int n_group, int *is_group) {
    const int nc = meta[MAX_LEVELS];
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        if (n_child[c] == 0 && count[c] > n_group) is_group[c] = 1;
    }
}

__global__ void k_compact_groups(const int *meta, const int *is_group, const int *off, int *group_cell) {
    const int nc = meta[MAX_LEVELS];
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x)
        if (is_group[c]) group_cell[off[c]] = c;
}

constexpr int GQ_WARPS = 2;
constexpr int GQCAP = 2048;   // ring buffer of opened cells per warp

// Breadth-first walk, four opened cells per iteration (eight lanes each).
// Order (shared with the oracle's or_grav_walk): cells are opened in FIFO
// order starting at the root; an opened leaf appends its particles to EPJ;
// an opened internal cell appends its unopened children to SPJ and its
// opened children to the queue, both in octant order.
template <bool FILL>
__global__ void __launch_bounds__(GQ_WARPS * 32)
k_grav_lists(int ng, const int *__restrict__ group_cell, const double *__restrict__ x,
             const double *__restrict__ y, const double *__restrict__ z, const int4 *__restrict__ cinfo,
             const int *__restrict__ clevel, const double4 *__restrict__ com, const double *__restrict__ rb_all,
             const int *__restrict__ prun, int *n_epj, int *n_spj, const int *off_epj, const int *off_spj, int *epj,
             int *spj, int *err) {
    __shared__ int s_q[GQ_WARPS][GQCAP];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = blockIdx.x * GQ_WARPS + warp;
    if (g >= ng) return;
    const int4 gi = cinfo[group_cell[g]];
    const int s = gi.z, cnt = gi.w;
    const int root = prun[s];   // the group's run: its octree root and opening radii
    const double *rb = rb_all + (int64_t)root * RB_STRIDE;
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int k = lane; k < cnt; k += 32) {
        const double p[3] = {x[s + k], y[s + k], z[s + k]};
        for (int d = 0; d < 3; ++d) {
            lo[d] = fmin(lo[d], p[d]);
            hi[d] = fmax(hi[d], p[d]);
        }
    }
    for (int d = 0; d < 3; ++d) {
        lo[d] = warp_min_d(lo[d]);
        hi[d] = warp_max_d(hi[d]);
    }
    int *Q = s_q[warp];
    int ne = 0, ns = 0;
    const int be = FILL ? off_epj[g] : 0, bs = FILL ? off_spj[g] : 0;
    if (lane == 0) Q[0] = root;
    int head = 0, tail = 1;
    const int q = lane >> 3, k = lane & 7;
    const unsigned below = (1u << lane) - 1u;
    __syncwarp();
    while (head < tail) {
        const int nproc = min(4, tail - head);
        const bool act = q < nproc;
        const int c = act ? Q[(head + q) & (GQCAP - 1)] : 0;
        const int4 ci = cinfo[c];                       // first_child, n_child, start, count
        const bool leaf = act && ci.y == 0;
        // opened leaves, in queue order
        for (int qq = 0; qq < nproc; ++qq) {
            const int cs = __shfl_sync(FULL, ci.z, qq * 8), ct = __shfl_sync(FULL, ci.w, qq * 8);
            const int lf = __shfl_sync(FULL, (int)leaf, qq * 8);
            if (lf) {
                if (FILL)
                    for (int t = lane; t < ct; t += 32) epj[be + ne + t] = cs + t;
                ne += ct;
            }
        }
        bool near = false, far = false;
        int ch = 0;
        if (act && !leaf && k < ci.y) {
            ch = ci.x + k;
            const double4 cm = com[ch];
            const double p[3] = {cm.x, cm.y, cm.z};
            double dd[3];
            for (int d = 0; d < 3; ++d)
                dd[d] = (p[d] < lo[d]) ? __dsub_rn(lo[d], p[d]) : ((p[d] > hi[d]) ? __dsub_rn(p[d], hi[d]) : 0.0);
            const double d2 =
                __dadd_rn(__dadd_rn(__dmul_rn(dd[0], dd[0]), __dmul_rn(dd[1], dd[1])), __dmul_rn(dd[2], dd[2]));
            near = d2 <= rb[8 + clevel[ch]];
            far = !near;
        }
        const unsigned nmask = __ballot_sync(FULL, near);
        const unsigned fmask = __ballot_sync(FULL, far);
        if (FILL && far) spj[bs + ns + __popc(fmask & below)] = ch;
        ns += __popc(fmask);
        const int nn = __popc(nmask);
        if (tail - head - nproc + nn > GQCAP) {
            if (lane == 0) atomicOr(err, ERR_GRAV_OVERFLOW);
            break;
        }
        __syncwarp();
        if (near) Q[(tail + __popc(nmask & below)) & (GQCAP - 1)] = ch;
        tail += nn;
        head += nproc;
        __syncwarp();
    }
    if (!FILL && lane == 0) {
        n_epj[g] = ne;
        n_spj[g] = ns;
    }
}


}  // namespace sph

using namespace sph;

template <class T>
static int dalloc_l(sph_ctx *ctx, T **p, int64_t n) {
    if (*p) cudaFree(*p);
    *p = nullptr;
    if (n <= 0) n = 1;
    cudaError_t e = cudaMalloc((void **)p, sizeof(T) * (size_t)n);
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return sph_fail(ctx, SPH_ERR_OOM, "device allocation of %lld bytes failed", (long long)(sizeof(T) * n));
    }
    return SPH_OK;
}

int sph_build_grav_groups(sph_ctx *ctx) {
    GravLists &G = ctx->grav;
    Tree &t = ctx->tree;
    const int nc = t.n_cell_host;
    const int grid = 2 * ctx->num_sms;
    cudaStream_t st = ctx->stream;
    k_mark_groups<<<grid, 256, 0, st>>>(t.meta, t.count, t.parent, ctx->cfg.n_group, G.is_group); ++ctx->launches;
    k_mark_groups_fix<<<grid, 256, 0, st>>>(t.meta, t.count, t.parent, t.n_child, ctx->cfg.n_group, G.is_group); ++ctx->launches;
    SPH_TRY(sph_scan_exclusive(ctx, G.is_group, t.tmp_off, nullptr, nc, t.meta + META_NGROUP));
    if (G.cap_groups < nc) {
        const int64_t c = nc + nc / 4 + 64;
        SPH_TRY(dalloc_l(ctx, &G.group_cell, c));
        SPH_TRY(dalloc_l(ctx, &G.n_epj, c + 1));
        SPH_TRY(dalloc_l(ctx, &G.n_spj, c + 1));
        SPH_TRY(dalloc_l(ctx, &G.off_epj, c + 1));
        SPH_TRY(dalloc_l(ctx, &G.off_spj, c + 1));
        G.cap_groups = c;
    }
    k_compact_groups<<<grid, 256, 0, st>>>(t.meta, G.is_group, t.tmp_off, G.group_cell); ++ctx->launches;
    int *hs = (int *)ctx->host_scalars;
    SPH_CUDA(ctx, cudaMemcpyAsync(hs, t.meta + META_NGROUP, sizeof(int), cudaMemcpyDeviceToHost, st));
    SPH_CUDA(ctx, cudaStreamSynchronize(st));
    const int ng = hs[0];
    G.ng = ng;
    return SPH_OK;
}

int sph_build_grav_lists(sph_ctx *ctx) {
    SPH_TRY(sph_build_grav_groups(ctx));
    GravLists &G = ctx->grav;
    Tree &t = ctx->tree;
    cudaStream_t st = ctx->stream;
    const int ng = G.ng;
    int *hs = (int *)ctx->host_scalars;
    const int blocks = (ng + GQ_WARPS - 1) / GQ_WARPS;
    SPH_CUDA(ctx, cudaMemsetAsync(t.meta + META_ERR, 0, sizeof(int), st));
    k_grav_lists<false><<<blocks, GQ_WARPS * 32, 0, st>>>(ng, G.group_cell, FLD(ctx->F, SPH_X, ctx->cap),
                                                         FLD(ctx->F, SPH_Y, ctx->cap), FLD(ctx->F, SPH_Z, ctx->cap),
                                                         t.cinfo, t.level, t.com, t.rb, ctx->runs.prun, G.n_epj, G.n_spj, nullptr,
                                                         nullptr, nullptr, nullptr, t.meta + META_ERR); ++ctx->launches;
    SPH_TRY(sph_scan_exclusive(ctx, G.n_epj, G.off_epj, nullptr, ng, nullptr));
    SPH_TRY(sph_scan_exclusive(ctx, G.n_spj, G.off_spj, nullptr, ng, nullptr));
    SPH_CUDA(ctx, cudaMemcpyAsync(hs, G.off_epj + (ng - 1), sizeof(int), cudaMemcpyDeviceToHost, st));
    SPH_CUDA(ctx, cudaMemcpyAsync(hs + 1, G.n_epj + (ng - 1), sizeof(int), cudaMemcpyDeviceToHost, st));
    SPH_CUDA(ctx, cudaMemcpyAsync(hs + 2, G.off_spj + (ng - 1), sizeof(int), cudaMemcpyDeviceToHost, st));
    SPH_CUDA(ctx, cudaMemcpyAsync(hs + 3, G.n_spj + (ng - 1), sizeof(int), cudaMemcpyDeviceToHost, st));
    SPH_CUDA(ctx, cudaMemcpyAsync(hs + 4, t.meta + META_ERR, sizeof(int), cudaMemcpyDeviceToHost, st));
    SPH_CUDA(ctx, cudaStreamSynchronize(st));
    if (hs[4] & ERR_GRAV_OVERFLOW) return sph_fail(ctx, SPH_ERR_CAPACITY, "gravity walk stack overflow");
    const int64_t tot_e = (int64_t)hs[0] + hs[1], tot_s = (int64_t)hs[2] + hs[3];
    if (tot_e > 2000000000LL || tot_s > 2000000000LL)
        return sph_fail(ctx, SPH_ERR_CAPACITY, "gravity interaction lists exceed 2^31 entries");
    if (G.cap_epj < tot_e) {
        G.cap_epj = tot_e + tot_e / 4 + 1024;
        SPH_TRY(dalloc_l(ctx, &G.epj, G.cap_epj));
    }
    if (G.cap_spj < tot_s) {
        G.cap_spj = tot_s + tot_s / 4 + 1024;
        SPH_TRY(dalloc_l(ctx, &G.spj, G.cap_spj));
    }
    G.tot_epj = tot_e;
    G.tot_spj = tot_s;
    k_grav_lists<true><<<blocks, GQ_WARPS * 32, 0, st>>>(ng, G.group_cell, FLD(ctx->F, SPH_X, ctx->cap),
                                                        FLD(ctx->F, SPH_Y, ctx->cap), FLD(ctx->F, SPH_Z, ctx->cap),
                                                        t.cinfo, t.level, t.com, t.rb, ctx->runs.prun, G.n_epj, G.n_spj, G.off_epj,
                                                        G.off_spj, G.epj, G.spj, t.meta + META_ERR); ++ctx->launches;
    SPH_CUDA(ctx, cudaGetLastError());
    G.valid = true;
    G.counts_valid = true;
    return SPH_OK;
}
