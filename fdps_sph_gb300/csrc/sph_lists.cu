// Neighbour and interaction lists on the device.
//
// SPH (TreeForForceShort::Gather for density / derivative, ::Symmetry for
// hydro, main.cpp:79-81): each warp takes 32 consecutive particles in key
// order, walks the octree depth-first in octant order with the group's
// bounding box (so candidate leaves, and hence every list, come out in
// ascending particle order), and every lane keeps exactly the candidates
// with |x_j - x_i|^2 < (2.5 h_i)^2 (gather) or < max(2.5 h_i, 2.5 h_j)^2
// (symmetric).  The test runs in FP32 on group-relative coordinates with an
// explicit error band; candidates inside the band are decided by the exact
// FP64 test of the oracle (oracle/sph_oracle.c: or_sph_walk), so the lists
// are bit-identical to the oracle's.  Lists are stored ELL-style:
// nbr[k * pitch + i], cnt[i].
//
// Gravity (TreeForForceLong::Monopole, main.cpp:83,90): one warp per i-group
// (cells with <= n_group particles whose parent holds more) walks the tree
// with the group's FP64 bounding box; a child is opened iff
// dmin^2(box, com) <= (side / theta)^2, leaves give EPJ particle ranges and
// unopened cells give SPJ monopoles, both in the oracle's recursive order
// (or_grav_walk).  Counting pass, scan, filling pass.
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

// conservative squared box-box distance (rounded down) in FP32
__device__ __forceinline__ float box_gap2_rd(float4 a_lo, float4 a_hi, float glo_x, float glo_y, float glo_z,
                                             float ghi_x, float ghi_y, float ghi_z) {
    const float gx = fmaxf(0.0f, fmaxf(__fsub_rd(a_lo.x, ghi_x), __fsub_rd(glo_x, a_hi.x)));
    const float gy = fmaxf(0.0f, fmaxf(__fsub_rd(a_lo.y, ghi_y), __fsub_rd(glo_y, a_hi.y)));
    const float gz = fmaxf(0.0f, fmaxf(__fsub_rd(a_lo.z, ghi_z), __fsub_rd(glo_z, a_hi.z)));
    return __fadd_rd(__fadd_rd(__fmul_rd(gx, gx), __fmul_rd(gy, gy)), __fmul_rd(gz, gz));
}

template <int MODE>
__global__ void __launch_bounds__(LIST_WARPS * 32)
k_sph_lists(int n, const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ z,
            const double *__restrict__ h, TreeView T, int *__restrict__ nbr, int *__restrict__ cnt, int K,
            int64_t pitch, int *err, int *maxcnt) {
    __shared__ int s_stack[LIST_WARPS][STACK_CAP];
    __shared__ int s_cand[LIST_WARPS][CAND_CAP];
    __shared__ float4 s_tile[LIST_WARPS][32];
    __shared__ float s_h2[LIST_WARPS][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int chunk = blockIdx.x * LIST_WARPS + warp;
    if (chunk * 32 >= n) return;   // warp-uniform
    const int i = chunk * 32 + lane;
    const bool valid = i < n;
    const double xi = valid ? x[i] : 0.0, yi = valid ? y[i] : 0.0, zi = valid ? z[i] : 0.0;
    const double hi_ = valid ? h[i] : 0.0;
    const double Hi = __dmul_rn(SUPPORT, hi_);
    const double H2 = __dmul_rn(Hi, Hi);
    // group bounding box (FP64), centre and largest search radius
    const double lox = warp_min_d(valid ? xi : INFINITY), hix = warp_max_d(valid ? xi : -INFINITY);
    const double loy = warp_min_d(valid ? yi : INFINITY), hiy = warp_max_d(valid ? yi : -INFINITY);
    const double loz = warp_min_d(valid ? zi : INFINITY), hiz = warp_max_d(valid ? zi : -INFINITY);
    const double Rg = warp_max_d(valid ? Hi : 0.0);
    const double cx = 0.5 * (lox + hix), cy = 0.5 * (loy + hiy), cz = 0.5 * (loz + hiz);
    const float glx = __double2float_rd(lox), gly = __double2float_rd(loy), glz = __double2float_rd(loz);
    const float ghx = __double2float_ru(hix), ghy = __double2float_ru(hiy), ghz = __double2float_ru(hiz);
    const float Rgf = __double2float_ru(Rg);
    const float xri = (float)(xi - cx), yri = (float)(yi - cy), zri = (float)(zi - cz);
    const float L1i = fabsf(xri) + fabsf(yri) + fabsf(zri);
    const float H2f = (float)H2;
    int *stack = s_stack[warp];
    int *cand = s_cand[warp];
    int count = 0;
    int nc = 0;

    auto flush = [&]() {
        for (int b = 0; b < nc; b += 32) {
            const int k = b + lane;
            int j = -1;
            if (k < nc) {
                j = cand[k];
                const double xj = x[j], yj = y[j], zj = z[j];
                const float a = (float)(xj - cx), bb = (float)(yj - cy), c = (float)(zj - cz);
                s_tile[warp][lane] = make_float4(a, bb, c, fabsf(a) + fabsf(bb) + fabsf(c));
                if (MODE == 1) {
                    const double Hj = __dmul_rn(SUPPORT, h[j]);
                    s_h2[warp][lane] = (float)__dmul_rn(Hj, Hj);
                }
            }
            __syncwarp();
            const int tc = min(32, nc - b);
            for (int t = 0; t < tc; ++t) {
                const float4 q = s_tile[warp][t];
                const int jj = __shfl_sync(FULL, j, t);
                const float dx = q.x - xri, dy = q.y - yri, dz = q.z - zri;
                const float r2f = dx * dx + dy * dy + dz * dz;
                float thr = H2f;
                if (MODE == 1) thr = fmaxf(thr, s_h2[warp][t]);
                const float S = L1i + q.w;
                const float tol = 3.814697265625e-06f * S * S + 9.5367431640625e-07f * thr;  // 2^-18 S^2 + 2^-20 thr
                bool ok;
                if (r2f < thr - tol) {
                    ok = true;
                } else if (r2f > thr + tol) {
                    ok = false;
                } else {
                    // exact FP64 decision, identical to the oracle's
                    const double ex = __dsub_rn(x[jj], xi), ey = __dsub_rn(y[jj], yi), ez = __dsub_rn(z[jj], zi);
                    const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez));
                    ok = r2 < H2;
                    if (MODE == 1 && !ok) {
                        const double Hj = __dmul_rn(SUPPORT, h[jj]);
                        ok = r2 < __dmul_rn(Hj, Hj);
                    }
                }
                if (valid && ok) {
                    if (count < K) nbr[(int64_t)count * pitch + i] = jj;
                    ++count;
                }
            }
            __syncwarp();
        }
        nc = 0;
    };

    // root test
    int sp = 0;
    {
        const float4 a = T.blo[0], b = T.bhi[0];
        float R = Rgf;
        if (MODE == 1) R = fmaxf(R, __fmul_ru(2.5f, b.w));
        const float d2 = box_gap2_rd(a, b, glx, gly, glz, ghx, ghy, ghz);
        if (d2 < __fmul_ru(R, R)) {
            if (lane == 0) stack[0] = 0;
            sp = 1;
        }
        __syncwarp();
    }
    while (sp > 0) {
        const int c = stack[--sp];
        __syncwarp();
        const int nch = T.n_child[c];
        if (nch == 0) {
            const int s = T.start[c], ct = T.count[c];
            for (int b0 = 0; b0 < ct; b0 += 32) {
                if (nc + 32 > CAND_CAP) flush();
                const int k = b0 + lane;
                if (k < ct) cand[nc + lane] = s + k;
                nc += min(32, ct - b0);
                __syncwarp();
            }
        } else {
            const int f = T.first_child[c];
            bool ok = false;
            if (lane < nch) {
                const float4 a = T.blo[f + lane], b = T.bhi[f + lane];
                float R = Rgf;
                if (MODE == 1) R = fmaxf(R, __fmul_ru(2.5f, b.w));
                const float d2 = box_gap2_rd(a, b, glx, gly, glz, ghx, ghy, ghz);
                ok = d2 < __fmul_ru(R, R);
            }
            const unsigned mask = __ballot_sync(FULL, ok);
            const int np = __popc(mask);
            if (sp + np > STACK_CAP) {
                if (lane == 0) atomicOr(err, ERR_SPH_LIST_OVERFLOW);
                break;
            }
            if (ok) stack[sp + (np - 1 - __popc(mask & ((1u << lane) - 1u)))] = f + lane;
            sp += np;
            __syncwarp();
        }
    }
    flush();
    if (valid) {
        cnt[i] = count;
        if (count > K) atomicOr(err, ERR_SPH_LIST_OVERFLOW);
    }
    const int wm = warp_max_i(valid ? count : 0);
    if (lane == 0) atomicMax(maxcnt, wm);
}

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

constexpr int GSTACK = 256;
constexpr int SPJ_FLAG = 1 << 30;

template <bool FILL>
__global__ void __launch_bounds__(LIST_WARPS * 32)
k_grav_lists(int ng, const int *__restrict__ group_cell, const double *__restrict__ x,
             const double *__restrict__ y, const double *__restrict__ z, TreeView T, const double *__restrict__ rb,
             int *n_epj, int *n_spj, const int *off_epj, const int *off_spj, int *epj, int *spj, int *err) {
    __shared__ int s_stack[LIST_WARPS][GSTACK];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int g = blockIdx.x * LIST_WARPS + warp;
    if (g >= ng) return;
    const int gc = group_cell[g];
    const int s = T.start[gc], cnt = T.count[gc];
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
    int *stack = s_stack[warp];
    int ne = 0, ns = 0;
    const int be = FILL ? off_epj[g] : 0, bs = FILL ? off_spj[g] : 0;
    if (lane == 0) stack[0] = 0;
    int sp = 1;
    __syncwarp();
    while (sp > 0) {
        const int item = stack[--sp];
        __syncwarp();
        if (item & SPJ_FLAG) {
            if (FILL && lane == 0) spj[bs + ns] = item & ~SPJ_FLAG;
            ++ns;
            continue;
        }
        const int c = item;
        const int nch = T.n_child[c];
        if (nch == 0) {
            const int cs = T.start[c], ct = T.count[c];
            if (FILL)
                for (int k = lane; k < ct; k += 32) epj[be + ne + k] = cs + k;
            ne += ct;
            continue;
        }
        const int f = T.first_child[c];
        if (sp + nch > GSTACK) {
            if (lane == 0) atomicOr(err, ERR_GRAV_OVERFLOW);
            break;
        }
        if (lane < nch) {
            const int ch = f + lane;
            const double4 cm = T.com[ch];
            const double p[3] = {cm.x, cm.y, cm.z};
            double dd[3];
            for (int d = 0; d < 3; ++d)
                dd[d] = (p[d] < lo[d]) ? __dsub_rn(lo[d], p[d]) : ((p[d] > hi[d]) ? __dsub_rn(p[d], hi[d]) : 0.0);
            const double d2 =
                __dadd_rn(__dadd_rn(__dmul_rn(dd[0], dd[0]), __dmul_rn(dd[1], dd[1])), __dmul_rn(dd[2], dd[2]));
            const bool near = d2 <= rb[8 + T.level[ch]];
            stack[sp + (nch - 1 - lane)] = near ? ch : (ch | SPJ_FLAG);
        }
        sp += nch;
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

static TreeView tree_view(sph_ctx *ctx) {
    Tree &t = ctx->tree;
    return TreeView{t.start, t.count, t.first_child, t.n_child, t.level, t.blo, t.bhi, t.com};
}

int sph_build_sph_lists(sph_ctx *ctx, int mode) {
    const int n = (int)ctx->n;
    SphLists &L = ctx->lists[mode];
    const int64_t pitch = ((int64_t)n + 31) / 32 * 32;
    if (L.K == 0) L.K = 160;
    const int64_t cap = ctx->cap;
    const double *x = FLD(ctx->F, SPH_X, cap), *y = FLD(ctx->F, SPH_Y, cap), *z = FLD(ctx->F, SPH_Z, cap),
                 *h = FLD(ctx->F, SPH_SMTH, cap);
    int *meta = ctx->tree.meta;
    for (int attempt = 0; attempt < 3; ++attempt) {
        if (!L.nbr || L.pitch < pitch || L.K_alloc < L.K) {
            const int64_t p2 = std::max<int64_t>(pitch, L.pitch);
            SPH_TRY(dalloc_l(ctx, &L.nbr, (int64_t)L.K * p2));
            SPH_TRY(dalloc_l(ctx, &L.cnt, p2));
            L.pitch = p2;
            L.K_alloc = L.K;
        }
        SPH_CUDA(ctx, cudaMemsetAsync(meta + META_ERR, 0, sizeof(int), ctx->stream));
        SPH_CUDA(ctx, cudaMemsetAsync(meta + META_MAXCNT, 0, sizeof(int), ctx->stream));
        const int warps = (n + 31) / 32;
        const int blocks = (warps + LIST_WARPS - 1) / LIST_WARPS;
        if (mode == 0)
            k_sph_lists<0><<<blocks, LIST_WARPS * 32, 0, ctx->stream>>>(n, x, y, z, h, tree_view(ctx), L.nbr, L.cnt,
                                                                       L.K, L.pitch, meta + META_ERR,
                                                                       meta + META_MAXCNT);
        else
            k_sph_lists<1><<<blocks, LIST_WARPS * 32, 0, ctx->stream>>>(n, x, y, z, h, tree_view(ctx), L.nbr, L.cnt,
                                                                       L.K, L.pitch, meta + META_ERR,
                                                                       meta + META_MAXCNT);
        ++ctx->launches;
        SPH_CUDA(ctx, cudaGetLastError());
        int *hs = (int *)ctx->host_scalars;
        SPH_CUDA(ctx, cudaMemcpyAsync(hs, meta + META_ERR, 4 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        SPH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        const int errw = hs[0], maxc = hs[META_MAXCNT - META_ERR];
        if (errw & ERR_SPH_LIST_OVERFLOW) {
            if (maxc <= L.K) return sph_fail(ctx, SPH_ERR_CAPACITY, "SPH list walk stack overflow");
            L.K = maxc + maxc / 4 + 8;   // grow and rebuild
            continue;
        }
        L.valid = true;
        return SPH_OK;
    }
    return sph_fail(ctx, SPH_ERR_CAPACITY, "SPH neighbour list capacity could not be grown");
}

int sph_build_grav_lists(sph_ctx *ctx) {
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
    const int blocks = (ng + LIST_WARPS - 1) / LIST_WARPS;
    SPH_CUDA(ctx, cudaMemsetAsync(t.meta + META_ERR, 0, sizeof(int), st));
    k_grav_lists<false><<<blocks, LIST_WARPS * 32, 0, st>>>(ng, G.group_cell, FLD(ctx->F, SPH_X, ctx->cap),
                                                           FLD(ctx->F, SPH_Y, ctx->cap),
                                                           FLD(ctx->F, SPH_Z, ctx->cap), tree_view(ctx), t.rb,
                                                           G.n_epj, G.n_spj, nullptr, nullptr, nullptr, nullptr,
                                                           t.meta + META_ERR); ++ctx->launches;
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
    k_grav_lists<true><<<blocks, LIST_WARPS * 32, 0, st>>>(ng, G.group_cell, FLD(ctx->F, SPH_X, ctx->cap),
                                                          FLD(ctx->F, SPH_Y, ctx->cap), FLD(ctx->F, SPH_Z, ctx->cap),
                                                          tree_view(ctx), t.rb, G.n_epj, G.n_spj, G.off_epj,
                                                          G.off_spj, G.epj, G.spj, t.meta + META_ERR); ++ctx->launches;
    SPH_CUDA(ctx, cudaGetLastError());
    G.valid = true;
    return SPH_OK;
}
