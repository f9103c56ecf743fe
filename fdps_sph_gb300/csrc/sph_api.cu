// Device-resident whole-pass C ABI: context, EoS materials, upload /
// download, the step of main.cpp:125-173 and inspection calls.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <fstream>
#include <sstream>

#include "sph_internal.cuh"

using namespace sph;

int sph_fail(sph_ctx *ctx, int code, const char *fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (ctx) ctx->err = buf;
    return code;
}

// records an event ending timing segment `seg` (seg < 0: the start mark)
int time_mark(sph_ctx *ctx, int seg) {
    if (!ctx->timing || ctx->n_ev >= 64) return SPH_OK;
    ctx->mark_seg[ctx->n_ev] = seg;
    SPH_CUDA(ctx, cudaEventRecord(ctx->ev[ctx->n_ev++], ctx->stream));
    return SPH_OK;
}

namespace {

__global__ void k_iota32(int32_t *a, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = i;
}

// back to upload order: particle k of run r goes to base + slot[k], base = the run's first particle
// (all runs) or 0 (one run, k in [k0, k0 + n))
__global__ void k_unpermute(const double *F, double *F2, int64_t cap, int k0, int n, const int32_t *slot,
                            const int *prun, const int4 *info, const int64_t *id, int64_t *id2, const int32_t *mat,
                            int32_t *mat2) {
    const int k = k0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= k0 + n) return;
    const int dst = (info ? info[prun[k]].x : 0) + slot[k];
    for (int f = 0; f < SPH_NFIELD; ++f) F2[(int64_t)f * cap + dst] = F[(int64_t)f * cap + k];
    id2[dst] = id[k];
    mat2[dst] = mat[k];
}

// checks of an uploaded block: bad[0] = first particle whose mass is not positive and finite,
// bad[1] = first particle with an unset material (INT_MAX: none); part[b] = mass sum of block b's
// contiguous chunk through a fixed reduction tree (the same sum for the same block every time)
constexpr int CHECK_BLOCKS = 256;
__global__ void __launch_bounds__(256) k_check_block(int n, const double *__restrict__ mass,
                                                     const int32_t *__restrict__ mat,
                                                     const DevMaterial *__restrict__ mats, double *part, int *bad,
                                                     unsigned long long *mmax) {
    __shared__ double s[256];
    __shared__ unsigned long long s_mx[256];   // positive doubles order like their bit patterns
    unsigned long long mx = 0;
    const int chunk = (n + CHECK_BLOCKS - 1) / CHECK_BLOCKS;
    const int lo = blockIdx.x * chunk, hi = min(n, lo + chunk);
    double acc = 0.0;
    for (int i = lo + (int)threadIdx.x; i < hi; i += blockDim.x) {
        const double m = mass[i];
        if (!(m > 0.0) || !isfinite(m))
            atomicMin(&bad[0], i);
        else
            mx = max(mx, (unsigned long long)__double_as_longlong(m));
        const int q = mat[i];
        if (q < 0 || q >= MAX_MATERIALS || mats[q].kind < 0) atomicMin(&bad[1], i);
        acc += m;
    }
    s[threadIdx.x] = acc;
    s_mx[threadIdx.x] = mx;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            s[threadIdx.x] += s[threadIdx.x + w];
            s_mx[threadIdx.x] = max(s_mx[threadIdx.x], s_mx[threadIdx.x + w]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[blockIdx.x] = s[0];
        atomicMax(mmax, s_mx[0]);
    }
}

// k_unpermute for the fields in `mask` only, into a block in upload order
__global__ void k_unpermute_fields(const double *F, double *out, int64_t cap, int n, uint64_t mask,
                                   const int32_t *slot, const int *prun, const int4 *info) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int dst = (info ? info[prun[k]].x : 0) + slot[k];
    for (int f = 0; f < SPH_NFIELD; ++f)
        if ((mask >> f) & 1) out[(int64_t)f * cap + dst] = F[(int64_t)f * cap + k];
}

__global__ void k_fill32(int32_t *a, int n, int v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}

__global__ void k_iota64(int64_t *a, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = i;
}

// drops the particles [off, off + cnt) of run r; later runs move down and are renumbered
__global__ void k_remove_run(const double *F, double *F2, int64_t cap, int n_new, int off, int cnt, int r,
                             const int64_t *id, int64_t *id2, const int32_t *slot, int32_t *slot2, const int32_t *mat,
                             int32_t *mat2, const int *prun, int *prun2) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_new) return;
    const int src = k < off ? k : k + cnt;
    for (int f = 0; f < SPH_NFIELD; ++f) F2[(int64_t)f * cap + k] = F[(int64_t)f * cap + src];
    id2[k] = id[src];
    slot2[k] = slot[src];
    mat2[k] = mat[src];
    const int q = prun[src];
    prun2[k] = q > r ? q - 1 : q;
}

template <class T>
int dalloc(sph_ctx *ctx, T **p, int64_t n) {
    if (*p) cudaFree(*p);
    *p = nullptr;
    cudaError_t e = cudaMalloc((void **)p, sizeof(T) * (size_t)std::max<int64_t>(n, 1));
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return sph_fail(ctx, SPH_ERR_OOM, "device allocation of %lld bytes failed: %s",
                        (long long)(sizeof(T) * (size_t)n), cudaGetErrorString(e));
    }
    return SPH_OK;
}

int upload_materials(sph_ctx *ctx) {
    SPH_CUDA(ctx, cudaMemcpyAsync(ctx->mats_dev, ctx->mats_host, sizeof(ctx->mats_host), cudaMemcpyHostToDevice,
                                  ctx->stream));
    SPH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SPH_OK;
}

// accumulates the elapsed time between consecutive marks into their segments
int collect_timings(sph_ctx *ctx) {
    if (!ctx->timing || ctx->n_ev < 2) {
        ctx->n_ev = 0;
        return SPH_OK;
    }
    SPH_CUDA(ctx, cudaEventSynchronize(ctx->ev[ctx->n_ev - 1]));
    for (int k = 1; k < ctx->n_ev; ++k) {
        float ms = 0.0f;
        SPH_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev[k - 1], ctx->ev[k]));
        const int seg = ctx->mark_seg[k];
        if (seg >= 0 && seg < SEG_N) {
            ctx->seg_ms[seg] += ms;
            ctx->seg_calls[seg] += 1;
        }
    }
    ctx->n_ev = 0;
    return SPH_OK;
}

}  // namespace

// sph_step_download: the requested fields that the step has finished writing go to the host now,
// on the copy stream, while the step goes on (the state is in key order in F after the sort;
// nothing swaps the buffers again within the step)
int dl_milestone(sph_ctx *ctx, uint64_t final_fields) {
    const uint64_t send = ctx->dl_left & final_fields;
    if (!ctx->dl_host || !send) return SPH_OK;
    cudaEvent_t ev = ctx->dl_ev[ctx->dl_next++ & 7];
    SPH_CUDA(ctx, cudaEventRecord(ev, ctx->stream));
    SPH_CUDA(ctx, cudaStreamWaitEvent(ctx->copy_stream, ev, 0));
    const int n = (int)ctx->n;
    k_unpermute_fields<<<sph_div_up(n, 256), 256, 0, ctx->copy_stream>>>(ctx->F, ctx->dl_buf, ctx->dl_cap, n, send,
                                                                         ctx->slot, ctx->runs.prun, ctx->runs.info);
    ++ctx->launches;
    SPH_CUDA(ctx, cudaGetLastError());
    for (int f = 0; f < SPH_NFIELD;) {
        if (!((send >> f) & 1)) {
            ++f;
            continue;
        }
        int g = f;
        while (g < SPH_NFIELD && ((send >> g) & 1)) ++g;
        SPH_CUDA(ctx, cudaMemcpy2DAsync(ctx->dl_host + (int64_t)f * ctx->dl_ld, sizeof(double) * ctx->dl_ld,
                                        ctx->dl_buf + (int64_t)f * ctx->dl_cap, sizeof(double) * ctx->dl_cap,
                                        sizeof(double) * n, g - f, cudaMemcpyDeviceToHost, ctx->copy_stream));
        f = g;
    }
    ctx->dl_left &= ~send;
    return SPH_OK;
}

namespace {

#define FB(f) (1ull << (f))

// main.cpp:138-146 (positions fixed): sort + tree, density x n, EoS, derivative, hydro, gravity
int compute_forces(sph_ctx *ctx) {
    SPH_TRY(sph_sort_and_build(ctx));   // marks SEG_SORT and SEG_TREE
    // final from here on: positions, half-step velocities and energies (kick-drift, then sorted)
    SPH_TRY(dl_milestone(ctx, FB(SPH_X) | FB(SPH_Y) | FB(SPH_Z) | FB(SPH_VHX) | FB(SPH_VHY) | FB(SPH_VHZ) |
                                  FB(SPH_ENGHALF)));
    if (ctx->cfg.precision == SPH_PREC_MIXED) SPH_TRY(sph_pack_mixed(ctx));
    SPH_TRY(time_mark(ctx, SEG_NBR_PREP));
    if (ctx->cfg.precision == SPH_PREC_MIXED) {
        // all passes straight from the superset, with the same neighbour decisions as the exact list
        SPH_TRY(sph_density_fused(ctx));
    } else {
        for (int it = 0; it < ctx->cfg.n_dens_iter; ++it) {
            SPH_TRY(sph_build_sph_lists(ctx, 0));
            SPH_TRY(time_mark(ctx, SEG_DENS_LIST));
            SPH_TRY(sph_pass_density(ctx, 0));
            SPH_TRY(time_mark(ctx, SEG_DENS));
        }
    }
    SPH_TRY(sph_pass_eos(ctx));
    SPH_TRY(time_mark(ctx, SEG_EOS));
    SPH_TRY(dl_milestone(ctx, FB(SPH_DENS) | FB(SPH_SMTH) | FB(SPH_PRES) | FB(SPH_SNDS)));
    SPH_TRY(sph_build_sph_lists(ctx, 2));   // gather and symmetric lists of the final h, one pass
    SPH_TRY(time_mark(ctx, SEG_DRVT_LIST));
    SPH_TRY(sph_pass_derivative(ctx, 0));
    SPH_TRY(time_mark(ctx, SEG_DRVT));
    SPH_TRY(dl_milestone(ctx, FB(SPH_DIVV) | FB(SPH_ROTX) | FB(SPH_ROTY) | FB(SPH_ROTZ) | FB(SPH_GRADH) |
                                  FB(SPH_BAL)));
    SPH_TRY(time_mark(ctx, SEG_HYDRO_LIST));
    SPH_TRY(sph_pass_hydro(ctx, 0));
    SPH_TRY(time_mark(ctx, SEG_HYDRO));
    // the external damping (GI.h:458-465) adds to acc after this, at the end of the step
    SPH_TRY(dl_milestone(ctx, FB(SPH_ENGDOT) | FB(SPH_DT) |
                                  (ctx->cfg.ext_damp ? 0ull : FB(SPH_AX) | FB(SPH_AY) | FB(SPH_AZ))));
    if (ctx->cfg.self_gravity) {
        if (ctx->cfg.precision == SPH_PREC_MIXED) {
            SPH_TRY(time_mark(ctx, SEG_GRAV_LIST));   // no lists: the walk runs inside the force kernel
            SPH_TRY(sph_gravity_fused(ctx));
        } else {
            SPH_TRY(sph_build_grav_lists(ctx));
            SPH_TRY(time_mark(ctx, SEG_GRAV_LIST));
            SPH_TRY(sph_pass_gravity(ctx, 0));
        }
        SPH_TRY(time_mark(ctx, SEG_GRAV));
        SPH_TRY(dl_milestone(ctx, FB(SPH_GX) | FB(SPH_GY) | FB(SPH_GZ) | FB(SPH_POT)));
    }
    ctx->have_forces = true;
    return SPH_OK;
}

}  // namespace

// offsets, tiles and device tables of the runs (after the run set changed)
int sph_runs_layout(sph_ctx *ctx) {
    Runs &R = ctx->runs;
    R.off.assign(R.R, 0);
    std::vector<int4> info(R.R), tiles;
    int64_t o = 0;
    int T = 0;
    for (int r = 0; r < R.R; ++r) {
        R.off[r] = o;
        const int nt = (int)((R.n[r] + RUN_TILE - 1) / RUN_TILE);
        info[r] = make_int4((int)o, (int)R.n[r], T, nt);
        for (int k = 0; k < nt; ++k)
            tiles.push_back(make_int4((int)(o + (int64_t)k * RUN_TILE), (int)std::min<int64_t>(RUN_TILE, R.n[r] - (int64_t)k * RUN_TILE),
                                      256 * T + k, nt));
        o += R.n[r];
        T += nt;
    }
    R.T = T;
    if (R.R > R.cap_R) {
        const int c = std::max(16, std::max(R.R, 2 * R.cap_R));
        SPH_TRY(dalloc(ctx, &R.info, c));
        SPH_TRY(dalloc(ctx, &R.dt_dev, c));
        SPH_TRY(dalloc(ctx, &R.out, 8 * (int64_t)c));
        SPH_TRY(dalloc(ctx, &R.damp, c));
        SPH_TRY(dalloc(ctx, &R.fixd, c));
        R.cap_R = c;
    }
    if (T > R.cap_T) {
        const int c = std::max(64, std::max(T, R.cap_T + R.cap_T / 2));
        SPH_TRY(dalloc(ctx, &R.tiles, c));
        SPH_TRY(dalloc(ctx, &R.part, 8 * (int64_t)c));
        R.cap_T = c;
    }
    std::vector<int> fixd(R.R);
    R.fix_split = true;
    for (int r = 0; r < R.R; ++r) {
        fixd[r] = ctx->mexp - R.mexp[r];
        R.fix_split = R.fix_split && std::ldexp(R.mmax[r], R.mexp[r]) <= 15.0;
    }
    if (R.R > 0) {
        SPH_CUDA(ctx, cudaMemcpyAsync(R.info, info.data(), sizeof(int4) * R.R, cudaMemcpyHostToDevice, ctx->stream));
        SPH_CUDA(ctx, cudaMemcpyAsync(R.fixd, fixd.data(), sizeof(int) * R.R, cudaMemcpyHostToDevice, ctx->stream));
        SPH_CUDA(ctx, cudaMemcpyAsync(R.dt_dev, R.dt.data(), sizeof(double) * R.R, cudaMemcpyHostToDevice, ctx->stream));
    }
    if (T > 0)
        SPH_CUDA(ctx, cudaMemcpyAsync(R.tiles, tiles.data(), sizeof(int4) * T, cudaMemcpyHostToDevice, ctx->stream));
    SPH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));   // the host vectors are the copies' sources
    // derived per-step structures are rebuilt by the next step
    ctx->sup.valid = false;
    ctx->lists[0].valid = ctx->lists[1].valid = false;
    ctx->grav.valid = ctx->grav.counts_valid = false;
    return SPH_OK;
}

namespace {

// grows the particle arrays to hold `need`, keeping particles [0, n)
int grow_particles(sph_ctx *ctx, int64_t need) {
    if (need <= ctx->cap) return SPH_OK;
    const int64_t c = std::max<int64_t>(need, ctx->cap + ctx->cap / 2);
    const int64_t n = ctx->n;
    double *F = nullptr;
    int64_t *id = nullptr;
    int32_t *slot = nullptr, *mat = nullptr;
    int *prun = nullptr;
    SPH_TRY(dalloc(ctx, &F, (int64_t)SPH_NFIELD * c));
    SPH_TRY(dalloc(ctx, &id, c));
    SPH_TRY(dalloc(ctx, &slot, c));
    SPH_TRY(dalloc(ctx, &mat, c));
    SPH_TRY(dalloc(ctx, &prun, c));
    if (n > 0) {
        SPH_CUDA(ctx, cudaMemcpy2DAsync(F, sizeof(double) * c, ctx->F, sizeof(double) * ctx->cap, sizeof(double) * n,
                                        SPH_NFIELD, cudaMemcpyDeviceToDevice, ctx->stream));
        SPH_CUDA(ctx, cudaMemcpyAsync(id, ctx->id, sizeof(int64_t) * n, cudaMemcpyDeviceToDevice, ctx->stream));
        SPH_CUDA(ctx, cudaMemcpyAsync(slot, ctx->slot, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, ctx->stream));
        SPH_CUDA(ctx, cudaMemcpyAsync(mat, ctx->mat, sizeof(int32_t) * n, cudaMemcpyDeviceToDevice, ctx->stream));
        SPH_CUDA(ctx, cudaMemcpyAsync(prun, ctx->runs.prun, sizeof(int) * n, cudaMemcpyDeviceToDevice, ctx->stream));
        SPH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    for (void *p : {(void *)ctx->F, (void *)ctx->id, (void *)ctx->slot, (void *)ctx->mat, (void *)ctx->runs.prun})
        if (p) cudaFree(p);
    ctx->F = F;
    ctx->id = id;
    ctx->slot = slot;
    ctx->mat = mat;
    ctx->runs.prun = prun;
    SPH_TRY(dalloc(ctx, &ctx->F2, (int64_t)SPH_NFIELD * c));
    SPH_TRY(dalloc(ctx, &ctx->id2, c));
    SPH_TRY(dalloc(ctx, &ctx->slot2, c));
    SPH_TRY(dalloc(ctx, &ctx->mat2, c));
    SPH_TRY(dalloc(ctx, &ctx->runs.prun2, c));
    SPH_TRY(dalloc(ctx, &ctx->keys, c));
    for (float4 **p : {&ctx->xh, &ctx->xl, &ctx->vhf, &ctx->vlf})
        if (*p) {
            cudaFree(*p);
            *p = nullptr;
        }
    ctx->cap = c;
    return SPH_OK;
}

int find_run(sph_ctx *ctx, int64_t handle) {
    for (int r = 0; r < ctx->runs.R; ++r)
        if (ctx->runs.handle[r] == handle) return r;
    return -1;
}

// appends a block of particles as a new run
int append_run(sph_ctx *ctx, int64_t n, const double *fields, int64_t ld, const int64_t *id, const int32_t *material,
               double time, double dt, int flags, int64_t *handle) {
    if (n < 1 || n > 0x3fffffff || !fields || ld < n || ctx->n + n > 0x3fffffff)
        return sph_fail(ctx, SPH_ERR_ARG, "bad particle block (n=%lld)", (long long)n);
    if (!material && ctx->mats_host[0].kind < 0) return sph_fail(ctx, SPH_ERR_ARG, "material 0 is not set");
    if ((flags & SPH_UPLOAD_STEP_INPUTS) && (flags & SPH_UPLOAD_INIT_SMTH))
        return sph_fail(ctx, SPH_ERR_ARG, "SPH_UPLOAD_INIT_SMTH reads the density, which SPH_UPLOAD_STEP_INPUTS leaves out");
    const int64_t o = ctx->n;
    SPH_TRY(grow_particles(ctx, o + n));
    const int64_t c = ctx->cap;
    // field rows: all of them, or (SPH_UPLOAD_STEP_INPUTS) the ones a step reads or carries, the
    // others zeroed; consecutive rows go in one 2D copy
    const uint64_t want = (flags & SPH_UPLOAD_STEP_INPUTS) ? (uint64_t)SPH_STEP_INPUT_FIELDS : ~0ull;
    for (int f = 0; f < SPH_NFIELD;) {
        const bool in = (want >> f) & 1;
        int g = f;
        while (g < SPH_NFIELD && (((want >> g) & 1) != 0) == in) ++g;
        if (in)
            SPH_CUDA(ctx, cudaMemcpy2DAsync(ctx->F + (int64_t)f * c + o, sizeof(double) * c, fields + (int64_t)f * ld,
                                            sizeof(double) * ld, sizeof(double) * n, g - f, cudaMemcpyHostToDevice,
                                            ctx->stream));
        else
            SPH_CUDA(ctx, cudaMemset2DAsync(ctx->F + (int64_t)f * c + o, sizeof(double) * c, 0, sizeof(double) * n,
                                            g - f, ctx->stream));
        f = g;
    }
    if (id) {
        SPH_CUDA(ctx, cudaMemcpyAsync(ctx->id + o, id, sizeof(int64_t) * n, cudaMemcpyHostToDevice, ctx->stream));
    } else {
        k_iota64<<<sph_div_up(n, 256), 256, 0, ctx->stream>>>(ctx->id + o, (int)n); ++ctx->launches;
    }
    if (material) {
        SPH_CUDA(ctx, cudaMemcpyAsync(ctx->mat + o, material, sizeof(int32_t) * n, cudaMemcpyHostToDevice, ctx->stream));
    } else {
        SPH_CUDA(ctx, cudaMemsetAsync(ctx->mat + o, 0, sizeof(int32_t) * n, ctx->stream));
    }
    // masses and materials checked on the device, the mass summed in a fixed order
    // (scratch: CHECK_BLOCKS partial sums, the two first bad indices, the largest mass's bits)
    double *part = ctx->scratch_d;
    int *bad = (int *)(ctx->scratch_d + CHECK_BLOCKS);
    unsigned long long *mmax = (unsigned long long *)(ctx->scratch_d + CHECK_BLOCKS + 1);
    const int big[4] = {INT_MAX, INT_MAX, 0, 0};
    std::memcpy(ctx->host_scalars + CHECK_BLOCKS, big, sizeof(big));
    SPH_CUDA(ctx, cudaMemcpyAsync(bad, ctx->host_scalars + CHECK_BLOCKS, sizeof(big), cudaMemcpyHostToDevice,
                                  ctx->stream));
    k_check_block<<<CHECK_BLOCKS, 256, 0, ctx->stream>>>((int)n, ctx->F + (int64_t)SPH_MASS * c + o, ctx->mat + o,
                                                         ctx->mats_dev, part, bad, mmax); ++ctx->launches;
    SPH_CUDA(ctx, cudaGetLastError());
    SPH_CUDA(ctx, cudaMemcpyAsync(ctx->host_scalars, part, sizeof(double) * CHECK_BLOCKS + sizeof(big),
                                  cudaMemcpyDeviceToHost, ctx->stream));
    Runs &R = ctx->runs;
    k_iota32<<<sph_div_up(n, 256), 256, 0, ctx->stream>>>(ctx->slot + o, (int)n); ++ctx->launches;
    k_fill32<<<sph_div_up(n, 256), 256, 0, ctx->stream>>>(R.prun + o, (int)n, R.R); ++ctx->launches;
    SPH_CUDA(ctx, cudaGetLastError());
    SPH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    int badh[2];
    std::memcpy(badh, ctx->host_scalars + CHECK_BLOCKS, sizeof(badh));
    if (badh[0] != INT_MAX) {
        double mi = 0.0;
        SPH_CUDA(ctx, cudaMemcpy(&mi, ctx->F + (int64_t)SPH_MASS * c + o + badh[0], sizeof(double),
                                 cudaMemcpyDeviceToHost));
        return sph_fail(ctx, SPH_ERR_NONFINITE, "particle %d has mass %g", badh[0], mi);
    }
    if (badh[1] != INT_MAX) return sph_fail(ctx, SPH_ERR_ARG, "particle %d uses an unset material", badh[1]);
    double msum = 0.0;
    for (int b = 0; b < CHECK_BLOCKS; ++b) msum += ctx->host_scalars[b];
    // power of two close to 1 / mean mass (exact rescaling of the FP32 mass copies), fixed by the first run
    // the run's own mass scale, a power of two close to 1 / its mean mass; the context's is its
    // first run's (exact rescaling of the FP32 mass copies).  The density sums of a run are
    // rounded on its own scale, so a run gives the same sums alone and in any mix.
    const int mexp = -(int)std::lround(std::log2(msum / (double)n));
    if (o == 0) {
        ctx->mexp = mexp;
        ctx->mscale = std::ldexp(1.0, mexp);
    } else if (std::abs(mexp - ctx->mexp) > 60) {
        return sph_fail(ctx, SPH_ERR_ARG, "the run's mean particle mass is 2^%d times the first run's (at most 2^60)",
                        ctx->mexp - mexp);
    }
    double mmax_h;
    std::memcpy(&mmax_h, ctx->host_scalars + CHECK_BLOCKS + 1, sizeof(mmax_h));
    if (flags & SPH_UPLOAD_INIT_SMTH) {
        SPH_TRY(sph_init_smth(ctx, o, n));
        SPH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    const bool forces = (flags & SPH_UPLOAD_FORCES_VALID) && dt > 0.0;
    R.n.push_back(n);
    R.time.push_back(time);
    R.dt.push_back(forces ? dt : 0.0);
    R.steps.push_back(0);
    R.handle.push_back(R.next_handle++);
    R.fresh.push_back(forces ? 0 : 1);
    R.mexp.push_back(mexp);
    R.mmax.push_back(mmax_h);
    R.R += 1;
    ctx->n = o + n;
    if (handle) *handle = R.handle.back();
    return sph_runs_layout(ctx);
}

}  // namespace

extern "C" {

void sph_config_default(sph_config *cfg) {
    if (!cfg) return;
    std::memset(cfg, 0, sizeof(*cfg));
    cfg->theta = 0.5;
    cfg->n_leaf = 8;
    cfg->n_group = 256;
    cfg->n_dens_iter = 4;
    cfg->self_gravity = 1;
    cfg->ext_damp = 0;
    cfg->precision = SPH_PREC_FP64;
    cfg->ext_damp_tend = 5000.0;
    cfg->damping = 1.0;
    cfg->G = 6.67e-11;
    cfg->device = 0;
    cfg->mode = 1;
    cfg->mantle_entropy = 3.12432609e+03;   // main.cpp:116-117
    cfg->core_entropy = 3.12432609e+03;     // main.cpp:118-119
    cfg->entropy_grid = 120;                // EoS.h:250-251, 403-404
    cfg->entropy_abs = SPH_ENTROPY_ABS_INT;
}

int sph_ctx_create(const sph_config *cfg, sph_ctx **out) {
    if (!out) return SPH_ERR_ARG;
    *out = nullptr;
    sph_ctx *ctx = new (std::nothrow) sph_ctx();
    if (!ctx) return SPH_ERR_OOM;
    if (cfg) ctx->cfg = *cfg;
    else sph_config_default(&ctx->cfg);
    const sph_config &c = ctx->cfg;
    if (!(c.theta >= 0.0) || c.n_leaf < 1 || c.n_group < 1 || c.n_dens_iter < 1 || c.n_dens_iter > 64 ||
        (c.precision != SPH_PREC_FP64 && c.precision != SPH_PREC_MIXED) || (c.mode != 1 && c.mode != 2) ||
        c.entropy_grid < 1 || (c.entropy_abs != SPH_ENTROPY_ABS_INT && c.entropy_abs != SPH_ENTROPY_ABS_REAL) ||
        !std::isfinite(c.mantle_entropy) || !std::isfinite(c.core_entropy)) {
        delete ctx;
        return SPH_ERR_ARG;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0 || c.device < 0 || c.device >= ndev) {
        cudaGetLastError();
        delete ctx;
        return SPH_ERR_CUDA;
    }
    ctx->device = c.device;
    if (cudaSetDevice(ctx->device) != cudaSuccess ||
        cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, ctx->device) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete ctx;
        return SPH_ERR_CUDA;
    }
    for (int k = 0; k < MAX_MATERIALS; ++k) {
        std::memset(&ctx->mats_host[k], 0, sizeof(DevMaterial));
        ctx->mats_host[k].kind = -1;
    }
    for (int k = 0; k < 64; ++k) cudaEventCreate(&ctx->ev[k]);
    for (int k = 0; k < 8; ++k) cudaEventCreateWithFlags(&ctx->dl_ev[k], cudaEventDisableTiming);
    cudaEventCreate(&ctx->ev_begin);
    cudaEventCreate(&ctx->ev_end);
    if (cudaMalloc((void **)&ctx->mats_dev, sizeof(ctx->mats_host)) != cudaSuccess ||
        cudaMalloc((void **)&ctx->scratch_d, sizeof(double) * 8192) != cudaSuccess ||
        cudaMallocHost((void **)&ctx->host_scalars, sizeof(double) * 512) != cudaSuccess) {
        cudaGetLastError();
        sph_ctx_destroy(ctx);
        return SPH_ERR_OOM;
    }
    if (upload_materials(ctx) != SPH_OK) {
        sph_ctx_destroy(ctx);
        return SPH_ERR_CUDA;
    }
    *out = ctx;
    return SPH_OK;
}

int sph_ctx_destroy(sph_ctx *ctx) {
    if (!ctx) return SPH_OK;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
    void *ptrs[] = {ctx->F, ctx->F2, ctx->id, ctx->id2, ctx->slot, ctx->slot2, ctx->mat, ctx->mat2, ctx->keys,
                    ctx->scratch_d, ctx->xh, ctx->xl, ctx->vhf, ctx->vlf, ctx->mats_dev,
                    ctx->tree.start, ctx->tree.count, ctx->tree.level, ctx->tree.first_child, ctx->tree.n_child,
                    ctx->tree.parent, ctx->tree.mom, ctx->tree.com, ctx->tree.blo, ctx->tree.bhi,
                    ctx->tree.tmp_cnt, ctx->tree.tmp_off, ctx->tree.tmp_b, ctx->tree.meta, ctx->tree.rb,
                    ctx->sort.k0, ctx->sort.k1, ctx->sort.v0, ctx->sort.v1, ctx->sort.hist, ctx->sort.hoff,
                    ctx->lists[0].nbr, ctx->lists[0].cnt, ctx->lists[1].nbr, ctx->lists[1].cnt,
                    ctx->grav.group_cell, ctx->grav.is_group, ctx->grav.n_epj, ctx->grav.n_spj, ctx->grav.off_epj,
                    ctx->grav.off_spj, ctx->grav.epj, ctx->grav.spj, ctx->scan.part, ctx->scan.total,
                    ctx->sup.nbr, ctx->sup.cnt, ctx->sup.hsup, ctx->sup.pxh, ctx->sup.pxl, ctx->sup.H2f,
                    ctx->sup.units, ctx->tree.cinfo, ctx->sup.r2, ctx->sup.m, ctx->sup.vR, ctx->sup.cvR,
                    ctx->sup.umark, ctx->sup.uoff, ctx->sup.uidx, ctx->runs.prun, ctx->runs.prun2,
                    ctx->runs.tiles, ctx->runs.info, ctx->runs.dt_dev, ctx->runs.part, ctx->runs.out,
                    ctx->runs.damp, ctx->runs.fixd, ctx->sup.soff, ctx->sup.need, ctx->sup.uover, ctx->sup.npass, ctx->dl_buf};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    for (void *p : ctx->table_allocs) cudaFree(p);
    sph_entropy_free(ctx);
    for (auto &g : ctx->tree_graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    if (ctx->host_scalars) cudaFreeHost(ctx->host_scalars);
    for (int k = 0; k < 64; ++k)
        if (ctx->ev[k]) cudaEventDestroy(ctx->ev[k]);
    if (ctx->ev_begin) cudaEventDestroy(ctx->ev_begin);
    if (ctx->ev_end) cudaEventDestroy(ctx->ev_end);
    for (int k = 0; k < 8; ++k)
        if (ctx->dl_ev[k]) cudaEventDestroy(ctx->dl_ev[k]);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return SPH_OK;
}

const char *sph_last_error(const sph_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int sph_set_eos_table(sph_ctx *ctx, int material, const double *rho_axis, int n_rho, const double *u_axis, int n_u,
                      const double *pres, const double *snds) {
    if (!ctx) return SPH_ERR_ARG;
    if (material < 0 || material >= MAX_MATERIALS) return sph_fail(ctx, SPH_ERR_ARG, "material %d out of range", material);
    if (!rho_axis || !u_axis || !pres || !snds || n_rho < 1 || n_u < 1)
        return sph_fail(ctx, SPH_ERR_TABLE, "EoS table for material %d is empty", material);
    for (int k = 1; k < n_rho; ++k)
        if (!(rho_axis[k] > rho_axis[k - 1])) return sph_fail(ctx, SPH_ERR_TABLE, "density axis not ascending");
    for (int k = 1; k < n_u; ++k)
        if (!(u_axis[k] > u_axis[k - 1])) return sph_fail(ctx, SPH_ERR_TABLE, "energy axis not ascending");
    cudaSetDevice(ctx->device);
    const size_t plane = sizeof(double) * (size_t)n_rho * n_u;
    const size_t bytes = sizeof(double) * (n_rho + n_u) + 2 * plane;
    char *d = nullptr;
    if (cudaMalloc((void **)&d, bytes) != cudaSuccess) {
        cudaGetLastError();
        return sph_fail(ctx, SPH_ERR_OOM, "EoS table allocation");
    }
    ctx->table_allocs.push_back(d);
    double *dr = (double *)d, *du = dr + n_rho, *dp = du + n_u, *dc = dp + (size_t)n_rho * n_u;
    SPH_CUDA(ctx, cudaMemcpy(dr, rho_axis, sizeof(double) * n_rho, cudaMemcpyHostToDevice));
    SPH_CUDA(ctx, cudaMemcpy(du, u_axis, sizeof(double) * n_u, cudaMemcpyHostToDevice));
    SPH_CUDA(ctx, cudaMemcpy(dp, pres, plane, cudaMemcpyHostToDevice));
    SPH_CUDA(ctx, cudaMemcpy(dc, snds, plane, cudaMemcpyHostToDevice));
    DevMaterial &m = ctx->mats_host[material];
    std::memset(&m, 0, sizeof(m));
    m.kind = 0;
    m.n_rho = n_rho;
    m.n_u = n_u;
    m.rho = dr;
    m.u = du;
    m.pres = dp;
    m.snds = dc;
    ctx->m2_dirty = true;
    return upload_materials(ctx);
}

int sph_set_eos_entropy(sph_ctx *ctx, int material, const double *temp, const double *ent, const double *line_rho,
                        const double *line_u) {
    if (!ctx) return SPH_ERR_ARG;
    if (material < 0 || material >= MAX_MATERIALS) return sph_fail(ctx, SPH_ERR_ARG, "material %d out of range", material);
    DevMaterial &m = ctx->mats_host[material];
    if (m.kind != 0) return sph_fail(ctx, SPH_ERR_STATE, "material %d is not a table (set it first)", material);
    if (!temp || !ent) return sph_fail(ctx, SPH_ERR_TABLE, "material %d: temperature and entropy planes needed", material);
    const size_t nl = (size_t)m.n_rho * m.n_u;
    std::vector<double> lr(nl), lu(nl);
    std::vector<double> rho_ax(m.n_rho), u_ax(m.n_u);
    SPH_CUDA(ctx, cudaMemcpy(rho_ax.data(), m.rho, sizeof(double) * m.n_rho, cudaMemcpyDeviceToHost));
    SPH_CUDA(ctx, cudaMemcpy(u_ax.data(), m.u, sizeof(double) * m.n_u, cudaMemcpyDeviceToHost));
    for (size_t k = 0; k < nl; ++k) {
        lr[k] = line_rho ? line_rho[k] : rho_ax[k / m.n_u];
        lu[k] = line_u ? line_u[k] : u_ax[k % m.n_u];
    }
    // the binary searches of the mode-2 lookup stand for the reference's linear scans
    // (interpolation.h:131-182) only over non-decreasing line densities
    for (size_t k = 1; k < nl; ++k)
        if (!(lr[k] >= lr[k - 1]))
            return sph_fail(ctx, SPH_ERR_TABLE, "material %d: line densities not non-decreasing at line %zu", material, k);
    for (size_t k = 0; k < nl; ++k)
        if (!std::isfinite(lr[k]) || !std::isfinite(lu[k]) || !std::isfinite(ent[k]))
            return sph_fail(ctx, SPH_ERR_TABLE, "material %d: non-finite mode-2 column at line %zu", material, k);
    cudaSetDevice(ctx->device);
    const size_t plane = sizeof(double) * nl;
    char *d = nullptr;
    if (cudaMalloc((void **)&d, 4 * plane) != cudaSuccess) {
        cudaGetLastError();
        return sph_fail(ctx, SPH_ERR_OOM, "mode-2 table columns");
    }
    ctx->table_allocs.push_back(d);
    double *dt_ = (double *)d, *de = dt_ + nl, *dr = de + nl, *du = dr + nl;
    SPH_CUDA(ctx, cudaMemcpy(dt_, temp, plane, cudaMemcpyHostToDevice));
    SPH_CUDA(ctx, cudaMemcpy(de, ent, plane, cudaMemcpyHostToDevice));
    SPH_CUDA(ctx, cudaMemcpy(dr, lr.data(), plane, cudaMemcpyHostToDevice));
    SPH_CUDA(ctx, cudaMemcpy(du, lu.data(), plane, cudaMemcpyHostToDevice));
    m.temp = dt_;
    m.ent = de;
    m.line_rho = dr;
    m.line_u = du;
    ctx->m2_dirty = true;
    return upload_materials(ctx);
}

int sph_set_eos_ideal(sph_ctx *ctx, int material, double gamma) {
    if (!ctx) return SPH_ERR_ARG;
    if (material < 0 || material >= MAX_MATERIALS) return sph_fail(ctx, SPH_ERR_ARG, "material %d out of range", material);
    if (!(gamma > 1.0) || !std::isfinite(gamma)) return sph_fail(ctx, SPH_ERR_ARG, "ideal gas needs gamma > 1");
    DevMaterial &m = ctx->mats_host[material];
    std::memset(&m, 0, sizeof(m));
    m.kind = 2;
    m.par[0] = gamma;
    ctx->m2_dirty = true;
    return upload_materials(ctx);
}

// Reader with the semantics of EoS.h:121-221 (header "# n_rho n_u", '#' lines
// skipped, n_u rows per density block, columns rho u T P c_s S).
namespace {

// A rho-u text table as EoS.h:121-221 reads it: a header line "# n_rho n_u", comment lines
// skipped, n_u lines per density block, columns density, energy, temperature, pressure, sound
// speed and (optionally) entropy.  The density axis is column 0 of each block's first line, the
// energy axis column 1 of the first block's lines (EoS.h:218-221).
struct RhoUTable {
    int n_rho = 0, n_u = 0;
    bool six = true;   // every line has the entropy column
    std::vector<double> rho, u, cols[6];
};

int parse_rho_u(const char *path, RhoUTable &t, std::string &err) {
    std::ifstream in(path);
    char buf[512];
    if (!in.is_open()) {
        std::snprintf(buf, sizeof buf, "cannot open EoS table %s", path);
        err = buf;
        return SPH_ERR_TABLE;
    }
    std::string line;
    if (!std::getline(in, line)) {
        std::snprintf(buf, sizeof buf, "%s: empty file", path);
        err = buf;
        return SPH_ERR_TABLE;
    }
    {
        std::istringstream ss(line);
        std::string hash;
        ss >> hash >> t.n_rho >> t.n_u;
        if (hash != "#" || t.n_rho < 1 || t.n_u < 1) {
            std::snprintf(buf, sizeof buf, "%s: bad header", path);
            err = buf;
            return SPH_ERR_TABLE;
        }
    }
    const size_t nl = (size_t)t.n_rho * t.n_u;
    t.rho.assign(t.n_rho, 0.0);
    t.u.assign(t.n_u, 0.0);
    for (auto &c : t.cols) c.assign(nl, 0.0);
    size_t row = 0;
    while (std::getline(in, line)) {
        if (line.empty() || line[0] == '#') continue;
        std::istringstream ss(line);
        double v[6];
        int k = 0;
        while (k < 6 && (ss >> v[k])) ++k;
        if (k == 0) continue;
        if (k < 5) {
            std::snprintf(buf, sizeof buf, "%s: short row %zu", path, row);
            err = buf;
            return SPH_ERR_TABLE;
        }
        if (row >= nl) {
            std::snprintf(buf, sizeof buf, "%s: more rows than the header says", path);
            err = buf;
            return SPH_ERR_TABLE;
        }
        const size_t li = row / t.n_u, ci = row % t.n_u;
        if (ci == 0) t.rho[li] = v[0];
        if (li == 0) t.u[ci] = v[1];
        for (int c = 0; c < k; ++c) t.cols[c][row] = v[c];
        if (k < 6) t.six = false;
        ++row;
    }
    if (row != nl) {
        std::snprintf(buf, sizeof buf, "%s: %zu rows, header says %d x %d", path, row, t.n_rho, t.n_u);
        err = buf;
        return SPH_ERR_TABLE;
    }
    return SPH_OK;
}

thread_local std::string g_table_err;

}  // namespace

int sph_load_eos_table_file(sph_ctx *ctx, int material, const char *path) {
    if (!ctx || !path) return SPH_ERR_ARG;
    RhoUTable t;
    std::string err;
    const int rc = parse_rho_u(path, t, err);
    if (rc != SPH_OK) return sph_fail(ctx, rc, "%s", err.c_str());
    SPH_TRY(sph_set_eos_table(ctx, material, t.rho.data(), t.n_rho, t.u.data(), t.n_u, t.cols[3].data(),
                              t.cols[4].data()));
    if (!t.six) return SPH_OK;
    return sph_set_eos_entropy(ctx, material, t.cols[2].data(), t.cols[5].data(), t.cols[0].data(),
                               t.cols[1].data());
}

int sph_read_eos_table_file(const char *path, int *n_rho, int *n_u, double *rho, double *u, double *cols,
                            int *n_cols) {
    if (!path || !n_rho || !n_u) return SPH_ERR_ARG;
    RhoUTable t;
    const int rc = parse_rho_u(path, t, g_table_err);
    if (rc != SPH_OK) return rc;
    *n_rho = t.n_rho;
    *n_u = t.n_u;
    if (n_cols) *n_cols = t.six ? 6 : 5;
    const size_t nl = (size_t)t.n_rho * t.n_u;
    if (rho) std::memcpy(rho, t.rho.data(), sizeof(double) * t.n_rho);
    if (u) std::memcpy(u, t.u.data(), sizeof(double) * t.n_u);
    if (cols)
        for (int c = 0; c < 6; ++c) std::memcpy(cols + (size_t)c * nl, t.cols[c].data(), sizeof(double) * nl);
    return SPH_OK;
}

const char *sph_read_eos_table_error(void) { return g_table_err.c_str(); }

int sph_set_eos_tillotson(sph_ctx *ctx, int material, const double par[10]) {
    if (!ctx || !par) return SPH_ERR_ARG;
    if (material < 0 || material >= MAX_MATERIALS) return sph_fail(ctx, SPH_ERR_ARG, "material %d out of range", material);
    if (!(par[0] > 0.0) || !(par[1] > 0.0) || !(par[3] > par[2]))
        return sph_fail(ctx, SPH_ERR_ARG, "Tillotson parameters need rho0 > 0, u0 > 0, ucv > uiv");
    DevMaterial &m = ctx->mats_host[material];
    std::memset(&m, 0, sizeof(m));
    m.kind = 1;
    for (int k = 0; k < 10; ++k) m.par[k] = par[k];
    ctx->m2_dirty = true;
    return upload_materials(ctx);
}

int sph_upload(sph_ctx *ctx, int64_t n, const double *fields, int64_t ld, const int64_t *id, const int32_t *material,
               double time, double dt, int flags) {
    if (!ctx) return SPH_ERR_ARG;
    cudaSetDevice(ctx->device);
    // one run: the context's previous particles and runs are replaced
    Runs &R = ctx->runs;
    R.R = 0;
    R.n.clear();
    R.time.clear();
    R.dt.clear();
    R.steps.clear();
    R.handle.clear();
    R.fresh.clear();
    R.mexp.clear();
    R.mmax.clear();
    ctx->n = 0;
    ctx->uploaded = false;
    ctx->batch = false;
    SPH_TRY(append_run(ctx, n, fields, ld, id, material, time, dt, flags, nullptr));
    ctx->step = 0;
    ctx->uploaded = true;
    // SPH_UPLOAD_FORCES_VALID: acc / grav / eng_dot / dt in the block are the forces of this state
    ctx->have_forces = (flags & SPH_UPLOAD_FORCES_VALID) && dt > 0.0;
    return SPH_OK;
}

int sph_add_run(sph_ctx *ctx, int64_t n, const double *fields, int64_t ld, const int64_t *id, const int32_t *material,
                double time, double dt, int flags, int64_t *handle) {
    if (!ctx || !handle) return SPH_ERR_ARG;
    cudaSetDevice(ctx->device);
    if (!ctx->uploaded) {   // an empty context: the run set starts here
        ctx->runs.R = 0;
        ctx->n = 0;
    }
    SPH_TRY(append_run(ctx, n, fields, ld, id, material, time, dt, flags, handle));
    ctx->uploaded = true;
    ctx->batch = true;
    return SPH_OK;
}

int sph_remove_run(sph_ctx *ctx, int64_t handle) {
    if (!ctx) return SPH_ERR_ARG;
    const int r = find_run(ctx, handle);
    if (r < 0) return sph_fail(ctx, SPH_ERR_ARG, "no run %lld", (long long)handle);
    cudaSetDevice(ctx->device);
    Runs &R = ctx->runs;
    const int64_t cnt = R.n[r], off = R.off[r], n_new = ctx->n - cnt;
    if (n_new > 0) {
        k_remove_run<<<sph_div_up(n_new, 256), 256, 0, ctx->stream>>>(
            ctx->F, ctx->F2, ctx->cap, (int)n_new, (int)off, (int)cnt, r, ctx->id, ctx->id2, ctx->slot, ctx->slot2,
            ctx->mat, ctx->mat2, R.prun, R.prun2); ++ctx->launches;
        SPH_CUDA(ctx, cudaGetLastError());
        std::swap(ctx->F, ctx->F2);
        std::swap(ctx->id, ctx->id2);
        std::swap(ctx->slot, ctx->slot2);
        std::swap(ctx->mat, ctx->mat2);
        std::swap(R.prun, R.prun2);
    }
    R.n.erase(R.n.begin() + r);
    R.time.erase(R.time.begin() + r);
    R.dt.erase(R.dt.begin() + r);
    R.steps.erase(R.steps.begin() + r);
    R.handle.erase(R.handle.begin() + r);
    R.fresh.erase(R.fresh.begin() + r);
    R.mexp.erase(R.mexp.begin() + r);
    R.mmax.erase(R.mmax.begin() + r);
    R.R -= 1;
    ctx->n = n_new;
    if (R.R == 0) ctx->uploaded = false;
    return sph_runs_layout(ctx);
}

int sph_run_info(sph_ctx *ctx, int64_t handle, int64_t *n, double *time, double *dt, int64_t *steps) {
    if (!ctx) return SPH_ERR_ARG;
    const int r = find_run(ctx, handle);
    if (r < 0) return sph_fail(ctx, SPH_ERR_ARG, "no run %lld", (long long)handle);
    if (n) *n = ctx->runs.n[r];
    if (time) *time = ctx->runs.time[r];
    if (dt) *dt = ctx->runs.dt[r];
    if (steps) *steps = ctx->runs.steps[r];
    return SPH_OK;
}

int sph_list_runs(sph_ctx *ctx, int64_t *handles, int cap, int *n_runs) {
    if (!ctx || !n_runs) return SPH_ERR_ARG;
    *n_runs = ctx->runs.R;
    for (int r = 0; r < ctx->runs.R && r < cap; ++r)
        if (handles) handles[r] = ctx->runs.handle[r];
    return SPH_OK;
}

int sph_download_run(sph_ctx *ctx, int64_t handle, double *fields, int64_t ld, int64_t *id, int32_t *material) {
    if (!ctx) return SPH_ERR_ARG;
    const int r = find_run(ctx, handle);
    if (r < 0) return sph_fail(ctx, SPH_ERR_ARG, "no run %lld", (long long)handle);
    const Runs &R = ctx->runs;
    const int n = (int)R.n[r];
    if (!fields || ld < n) return sph_fail(ctx, SPH_ERR_ARG, "bad output block");
    cudaSetDevice(ctx->device);
    k_unpermute<<<sph_div_up(n, 256), 256, 0, ctx->stream>>>(ctx->F, ctx->F2, ctx->cap, (int)R.off[r], n, ctx->slot,
                                                             R.prun, nullptr, ctx->id, ctx->id2, ctx->mat,
                                                             ctx->mat2); ++ctx->launches;
    SPH_CUDA(ctx, cudaGetLastError());
    SPH_CUDA(ctx, cudaMemcpy2DAsync(fields, sizeof(double) * ld, ctx->F2, sizeof(double) * ctx->cap,
                                    sizeof(double) * n, SPH_NFIELD, cudaMemcpyDeviceToHost, ctx->stream));
    if (id) SPH_CUDA(ctx, cudaMemcpyAsync(id, ctx->id2, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, ctx->stream));
    if (material)
        SPH_CUDA(ctx, cudaMemcpyAsync(material, ctx->mat2, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, ctx->stream));
    SPH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SPH_OK;
}

int sph_run_diagnostics(sph_ctx *ctx, int64_t handle, double out[8]) {
    if (!ctx || !out) return SPH_ERR_ARG;
    const int r = find_run(ctx, handle);
    if (r < 0) return sph_fail(ctx, SPH_ERR_ARG, "no run %lld", (long long)handle);
    cudaSetDevice(ctx->device);
    std::vector<double> per(8 * (size_t)ctx->runs.R);
    SPH_TRY(sph_run_diag(ctx, per.data()));
    for (int k = 0; k < 8; ++k) out[k] = per[(size_t)r * 8 + k];
    return SPH_OK;
}

int sph_download_fields(sph_ctx *ctx, double *fields, int64_t ld, uint64_t field_mask, int64_t *id,
                        int32_t *material) {
    if (!ctx) return SPH_ERR_ARG;
    if (!ctx->uploaded) return sph_fail(ctx, SPH_ERR_STATE, "download before upload");
    if ((field_mask && !fields) || ld < ctx->n) return sph_fail(ctx, SPH_ERR_ARG, "bad output block");
    cudaSetDevice(ctx->device);
    const int n = (int)ctx->n;
    k_unpermute<<<sph_div_up(n, 256), 256, 0, ctx->stream>>>(ctx->F, ctx->F2, ctx->cap, 0, n, ctx->slot,
                                                             ctx->runs.prun, ctx->runs.info, ctx->id, ctx->id2,
                                                             ctx->mat, ctx->mat2); ++ctx->launches;
    SPH_CUDA(ctx, cudaGetLastError());
    // rows of consecutive requested fields in one 2D copy each
    for (int f = 0; f < SPH_NFIELD;) {
        if (!((field_mask >> f) & 1)) {
            ++f;
            continue;
        }
        int g = f;
        while (g < SPH_NFIELD && ((field_mask >> g) & 1)) ++g;
        SPH_CUDA(ctx, cudaMemcpy2DAsync(fields + (int64_t)f * ld, sizeof(double) * ld, ctx->F2 + (int64_t)f * ctx->cap,
                                        sizeof(double) * ctx->cap, sizeof(double) * n, g - f, cudaMemcpyDeviceToHost,
                                        ctx->stream));
        f = g;
    }
    if (id) SPH_CUDA(ctx, cudaMemcpyAsync(id, ctx->id2, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, ctx->stream));
    if (material)
        SPH_CUDA(ctx, cudaMemcpyAsync(material, ctx->mat2, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, ctx->stream));
    SPH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SPH_OK;
}

int sph_download(sph_ctx *ctx, double *fields, int64_t ld, int64_t *id, int32_t *material) {
    if (!ctx) return SPH_ERR_ARG;
    if (!fields) return sph_fail(ctx, SPH_ERR_ARG, "bad output block");
    return sph_download_fields(ctx, fields, ld, ~0ull, id, material);
}

int sph_prologue(sph_ctx *ctx) {
    if (!ctx) return SPH_ERR_ARG;
    if (!ctx->uploaded) return sph_fail(ctx, SPH_ERR_STATE, "prologue before upload");
    cudaSetDevice(ctx->device);
    ctx->n_ev = 0;
    SPH_TRY(time_mark(ctx, -1));
    SPH_TRY(compute_forces(ctx));
    SPH_TRY(sph_run_reduce_dt(ctx));           // main.cpp:103
    SPH_TRY(sph_ext_force(ctx));               // main.cpp:104
    SPH_TRY(time_mark(ctx, SEG_FINAL));
    SPH_TRY(collect_timings(ctx));
    SPH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int r = 0; r < ctx->runs.R; ++r) ctx->runs.fresh[r] = 0;
    ctx->have_forces = true;
    return SPH_OK;
}

// One loop iteration of main.cpp:125-173 for every run, each with its own dt.
// A run added since the last step (no forces yet) takes this step as its
// prologue: dt 0 in the kicks and the drift, then its forces and dt.
int sph_step(sph_ctx *ctx, int n_steps) {
    if (!ctx) return SPH_ERR_ARG;
    if (!ctx->uploaded) return sph_fail(ctx, SPH_ERR_STATE, "step before upload");
    if (!ctx->batch && !ctx->have_forces) return sph_fail(ctx, SPH_ERR_STATE, "step before prologue");
    cudaSetDevice(ctx->device);
    Runs &R = ctx->runs;
    for (int s = 0; s < n_steps; ++s) {
        ctx->n_ev = 0;
        SPH_TRY(time_mark(ctx, -1));
        bool fresh = false;
        for (int r = 0; r < R.R; ++r) fresh = fresh || R.fresh[r];
        std::vector<double> dt_step(R.dt);
        if (fresh) {
            for (int r = 0; r < R.R; ++r)
                if (R.fresh[r]) dt_step[r] = 0.0;
            SPH_CUDA(ctx, cudaMemcpyAsync(R.dt_dev, dt_step.data(), sizeof(double) * R.R, cudaMemcpyHostToDevice,
                                          ctx->stream));
        }
        SPH_TRY(sph_kick_drift_predict(ctx));       // main.cpp:126-131
        SPH_TRY(time_mark(ctx, SEG_KDP));
        for (int r = 0; r < R.R; ++r) R.time[r] += dt_step[r];   // main.cpp:132
        SPH_TRY(compute_forces(ctx));               // main.cpp:136-147
        SPH_TRY(sph_ext_force(ctx));                // main.cpp:148
        SPH_TRY(sph_final_kick(ctx));               // main.cpp:149-153
        if (ctx->cfg.mode == 2) {                   // main.cpp:155-158
            SPH_TRY(time_mark(ctx, SEG_FINAL));
            SPH_TRY(sph_entropy_step(ctx));
            SPH_TRY(time_mark(ctx, SEG_ENTROPY));
        }
        SPH_TRY(sph_run_reduce_dt(ctx));            // main.cpp:160
        if (ctx->cfg.mode == 2) SPH_TRY(sph_entropy_check(ctx));
        SPH_TRY(time_mark(ctx, SEG_FINAL));
        SPH_TRY(collect_timings(ctx));
        for (int r = 0; r < R.R; ++r) {
            if (R.fresh[r]) R.fresh[r] = 0;
            else R.steps[r] += 1;
        }
        ctx->step += 1;
        if (fresh) SPH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));   // dt_step is the copy's source
    }
    ctx->have_forces = true;
    return SPH_OK;
}

int sph_step_download(sph_ctx *ctx, double *fields, int64_t ld, uint64_t field_mask) {
    if (!ctx) return SPH_ERR_ARG;
    if (!ctx->uploaded) return sph_fail(ctx, SPH_ERR_STATE, "step before upload");
    if ((field_mask && !fields) || ld < ctx->n) return sph_fail(ctx, SPH_ERR_ARG, "bad output block");
    cudaSetDevice(ctx->device);
    if (ctx->dl_cap < ctx->cap) {
        if (ctx->dl_buf) cudaFree(ctx->dl_buf);
        ctx->dl_buf = nullptr;
        ctx->dl_cap = 0;
        if (cudaMalloc((void **)&ctx->dl_buf, sizeof(double) * SPH_NFIELD * (size_t)ctx->cap) != cudaSuccess) {
            cudaGetLastError();
            return sph_fail(ctx, SPH_ERR_OOM, "download staging block");
        }
        ctx->dl_cap = ctx->cap;
    }
    // the copy stream must not run ahead into staging rows an earlier call is still reading
    SPH_CUDA(ctx, cudaStreamSynchronize(ctx->copy_stream));
    ctx->dl_host = fields;
    ctx->dl_ld = ld;
    ctx->dl_left = field_mask & ((1ull << SPH_NFIELD) - 1);
    int rc = sph_step(ctx, 1);
    if (rc == SPH_OK) rc = dl_milestone(ctx, ~0ull);   // what the end of the step wrote
    ctx->dl_host = nullptr;
    ctx->dl_left = 0;
    const cudaError_t e = cudaStreamSynchronize(ctx->copy_stream);
    if (rc != SPH_OK) return rc;
    if (e != cudaSuccess) return sph_fail(ctx, SPH_ERR_CUDA, "download stream: %s", cudaGetErrorString(e));
    return SPH_OK;
}

int sph_get_time(const sph_ctx *ctx, double *time, double *dt, int64_t *step) {
    if (!ctx) return SPH_ERR_ARG;
    // the first run (the one of sph_upload)
    if (time) *time = ctx->runs.R ? ctx->runs.time[0] : 0.0;
    if (dt) *dt = ctx->runs.R ? ctx->runs.dt[0] : 0.0;
    if (step) *step = ctx->step;
    return SPH_OK;
}

int sph_diagnostics(sph_ctx *ctx, double out[8]) {
    if (!ctx || !out) return SPH_ERR_ARG;
    if (!ctx->uploaded) return sph_fail(ctx, SPH_ERR_STATE, "diagnostics before upload");
    cudaSetDevice(ctx->device);
    return sph_diag(ctx, out);
}

int sph_run_pass(sph_ctx *ctx, int pass) {
    if (!ctx) return SPH_ERR_ARG;
    if (!ctx->uploaded) return sph_fail(ctx, SPH_ERR_STATE, "pass before upload");
    cudaSetDevice(ctx->device);
    switch (pass) {
        case 0:
            SPH_TRY(sph_sort_and_build(ctx));
            if (ctx->cfg.precision == SPH_PREC_MIXED) SPH_TRY(sph_pack_mixed(ctx));
            break;
        case 1: SPH_TRY(sph_pass_density(ctx, 1)); break;
        case 2: SPH_TRY(sph_pass_eos(ctx)); break;
        case 3: SPH_TRY(sph_pass_derivative(ctx, 1)); break;
        case 4: SPH_TRY(sph_pass_hydro(ctx, 1)); break;
        case 5: SPH_TRY(sph_pass_gravity(ctx, 1)); break;
        default: return sph_fail(ctx, SPH_ERR_ARG, "unknown pass %d", pass);
    }
    SPH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SPH_OK;
}

int sph_get_order(sph_ctx *ctx, int32_t *slot, uint64_t *keys) {
    if (!ctx) return SPH_ERR_ARG;
    if (!ctx->uploaded) return sph_fail(ctx, SPH_ERR_STATE, "no particles");
    cudaSetDevice(ctx->device);
    if (slot) SPH_CUDA(ctx, cudaMemcpy(slot, ctx->slot, sizeof(int32_t) * ctx->n, cudaMemcpyDeviceToHost));
    if (keys) SPH_CUDA(ctx, cudaMemcpy(keys, ctx->keys, sizeof(uint64_t) * ctx->n, cudaMemcpyDeviceToHost));
    return SPH_OK;
}

int sph_get_neighbors(sph_ctx *ctx, int mode, int64_t k, int32_t *out, int64_t cap, int64_t *n) {
    if (!ctx || mode < 0 || mode > 1 || !n) return SPH_ERR_ARG;
    const SphLists &L = ctx->lists[mode];
    if (!L.valid) return sph_fail(ctx, SPH_ERR_STATE, "no list of mode %d", mode);
    if (k < 0 || k >= ctx->n) return sph_fail(ctx, SPH_ERR_ARG, "particle index out of range");
    cudaSetDevice(ctx->device);
    int c = 0;
    SPH_CUDA(ctx, cudaMemcpy(&c, L.cnt + k, sizeof(int), cudaMemcpyDeviceToHost));
    *n = c;
    const int64_t m = std::min<int64_t>(c, cap);
    const int64_t m0 = std::min<int64_t>(m, L.K);   // the row; the rest is in the particle's spill range
    if (out && m0 > 0)
        SPH_CUDA(ctx, cudaMemcpy(out, L.nbr + (int64_t)k * L.pitch, sizeof(int32_t) * m0, cudaMemcpyDeviceToHost));
    if (out && m > m0) {
        const RowMap rm = ctx->sup.map();
        if (!rm.soff) return sph_fail(ctx, SPH_ERR_STATE, "row of particle %lld has no spill range", (long long)k);
        int so = 0;
        SPH_CUDA(ctx, cudaMemcpy(&so, rm.soff + k, sizeof(int), cudaMemcpyDeviceToHost));
        SPH_CUDA(ctx, cudaMemcpy(out + m0, L.nbr + rm.main + so, sizeof(int32_t) * (m - m0), cudaMemcpyDeviceToHost));
    }
    return SPH_OK;
}

int sph_get_tree(sph_ctx *ctx, int64_t *n_cell, int32_t *start, int32_t *count, int32_t *level, int32_t *n_child,
                 double *com_mass) {
    if (!ctx || !n_cell) return SPH_ERR_ARG;
    cudaSetDevice(ctx->device);
    const int nc = ctx->tree.n_cell_host;
    *n_cell = nc;
    const Tree &t = ctx->tree;
    if (start) SPH_CUDA(ctx, cudaMemcpy(start, t.start, sizeof(int) * nc, cudaMemcpyDeviceToHost));
    if (count) SPH_CUDA(ctx, cudaMemcpy(count, t.count, sizeof(int) * nc, cudaMemcpyDeviceToHost));
    if (level) SPH_CUDA(ctx, cudaMemcpy(level, t.level, sizeof(int) * nc, cudaMemcpyDeviceToHost));
    if (n_child) SPH_CUDA(ctx, cudaMemcpy(n_child, t.n_child, sizeof(int) * nc, cudaMemcpyDeviceToHost));
    if (com_mass) SPH_CUDA(ctx, cudaMemcpy(com_mass, t.com, sizeof(double4) * nc, cudaMemcpyDeviceToHost));
    return SPH_OK;
}

int sph_get_grav_list(sph_ctx *ctx, int64_t g, int64_t *n_group, int32_t *epj, int64_t cap_epj, int64_t *n_epj,
                      int32_t *spj_level, int32_t *spj_start, int64_t cap_spj, int64_t *n_spj, int32_t *group_start,
                      int32_t *group_count) {
    if (!ctx) return SPH_ERR_ARG;
    const GravLists &G = ctx->grav;
    if (!G.valid) return sph_fail(ctx, SPH_ERR_STATE, "no gravity lists");
    if (n_group) *n_group = G.ng;
    if (g < 0) return SPH_OK;
    if (g >= G.ng) return sph_fail(ctx, SPH_ERR_ARG, "group index out of range");
    cudaSetDevice(ctx->device);
    int ne = 0, ns = 0, oe = 0, os = 0, gc = 0;
    SPH_CUDA(ctx, cudaMemcpy(&ne, G.n_epj + g, sizeof(int), cudaMemcpyDeviceToHost));
    SPH_CUDA(ctx, cudaMemcpy(&ns, G.n_spj + g, sizeof(int), cudaMemcpyDeviceToHost));
    SPH_CUDA(ctx, cudaMemcpy(&oe, G.off_epj + g, sizeof(int), cudaMemcpyDeviceToHost));
    SPH_CUDA(ctx, cudaMemcpy(&os, G.off_spj + g, sizeof(int), cudaMemcpyDeviceToHost));
    SPH_CUDA(ctx, cudaMemcpy(&gc, G.group_cell + g, sizeof(int), cudaMemcpyDeviceToHost));
    if (n_epj) *n_epj = ne;
    if (n_spj) *n_spj = ns;
    if (group_start) SPH_CUDA(ctx, cudaMemcpy(group_start, ctx->tree.start + gc, sizeof(int), cudaMemcpyDeviceToHost));
    if (group_count) SPH_CUDA(ctx, cudaMemcpy(group_count, ctx->tree.count + gc, sizeof(int), cudaMemcpyDeviceToHost));
    if (epj && ne > 0)
        SPH_CUDA(ctx, cudaMemcpy(epj, G.epj + oe, sizeof(int) * std::min<int64_t>(ne, cap_epj), cudaMemcpyDeviceToHost));
    if ((spj_level || spj_start) && ns > 0) {
        const int m = (int)std::min<int64_t>(ns, cap_spj);
        std::vector<int> cells(m);
        SPH_CUDA(ctx, cudaMemcpy(cells.data(), G.spj + os, sizeof(int) * m, cudaMemcpyDeviceToHost));
        for (int k = 0; k < m; ++k) {
            if (spj_level) SPH_CUDA(ctx, cudaMemcpy(spj_level + k, ctx->tree.level + cells[k], sizeof(int), cudaMemcpyDeviceToHost));
            if (spj_start) SPH_CUDA(ctx, cudaMemcpy(spj_start + k, ctx->tree.start + cells[k], sizeof(int), cudaMemcpyDeviceToHost));
        }
    }
    return SPH_OK;
}

int sph_get_grav_lists(sph_ctx *ctx, int64_t *n_group, int64_t *n_epj_total, int64_t *n_spj_total,
                       int32_t *group_start, int32_t *group_count, int32_t *epj_off, int32_t *epj_len, int32_t *epj,
                       int32_t *spj_off, int32_t *spj_len, int32_t *spj_cell) {
    if (!ctx || !n_group || !n_epj_total || !n_spj_total) return SPH_ERR_ARG;
    const GravLists &G = ctx->grav;
    if (!G.valid) return sph_fail(ctx, SPH_ERR_STATE, "no gravity lists (run an FP64 gravity pass first)");
    cudaSetDevice(ctx->device);
    const int ng = G.ng;
    *n_group = ng;
    std::vector<int> oe(ng), ne(ng), os(ng), ns(ng);
    if (ng > 0) {
        SPH_CUDA(ctx, cudaMemcpy(oe.data(), G.off_epj, sizeof(int) * ng, cudaMemcpyDeviceToHost));
        SPH_CUDA(ctx, cudaMemcpy(ne.data(), G.n_epj, sizeof(int) * ng, cudaMemcpyDeviceToHost));
        SPH_CUDA(ctx, cudaMemcpy(os.data(), G.off_spj, sizeof(int) * ng, cudaMemcpyDeviceToHost));
        SPH_CUDA(ctx, cudaMemcpy(ns.data(), G.n_spj, sizeof(int) * ng, cudaMemcpyDeviceToHost));
    }
    const int64_t te = ng ? (int64_t)oe[ng - 1] + ne[ng - 1] : 0, ts = ng ? (int64_t)os[ng - 1] + ns[ng - 1] : 0;
    *n_epj_total = te;
    *n_spj_total = ts;
    if (epj_off) std::memcpy(epj_off, oe.data(), sizeof(int) * ng);
    if (epj_len) std::memcpy(epj_len, ne.data(), sizeof(int) * ng);
    if (spj_off) std::memcpy(spj_off, os.data(), sizeof(int) * ng);
    if (spj_len) std::memcpy(spj_len, ns.data(), sizeof(int) * ng);
    if (epj && te > 0) SPH_CUDA(ctx, cudaMemcpy(epj, G.epj, sizeof(int) * te, cudaMemcpyDeviceToHost));
    if (spj_cell && ts > 0) SPH_CUDA(ctx, cudaMemcpy(spj_cell, G.spj, sizeof(int) * ts, cudaMemcpyDeviceToHost));
    if ((group_start || group_count) && ng > 0) {
        const int nc = ctx->tree.n_cell_host;
        std::vector<int> gc(ng), st(nc), ct(nc);
        SPH_CUDA(ctx, cudaMemcpy(gc.data(), G.group_cell, sizeof(int) * ng, cudaMemcpyDeviceToHost));
        SPH_CUDA(ctx, cudaMemcpy(st.data(), ctx->tree.start, sizeof(int) * nc, cudaMemcpyDeviceToHost));
        SPH_CUDA(ctx, cudaMemcpy(ct.data(), ctx->tree.count, sizeof(int) * nc, cudaMemcpyDeviceToHost));
        for (int g = 0; g < ng; ++g) {
            if (group_start) group_start[g] = st[gc[g]];
            if (group_count) group_count[g] = ct[gc[g]];
        }
    }
    return SPH_OK;
}

int sph_get_timings(sph_ctx *ctx, double *ms, int cap, int *n) {
    if (!ctx) return SPH_ERR_ARG;
    if (cap < 0) {   // -1: switch event timing on and reset, -2: off, -3: reset
        if (cap == -1) ctx->timing = true;
        if (cap == -2) ctx->timing = false;
        for (int k = 0; k < 16; ++k) {
            ctx->seg_ms[k] = 0.0;
            ctx->seg_calls[k] = 0;
        }
        return SPH_OK;
    }
    const int m = std::min(cap, (int)SEG_N);
    for (int k = 0; k < m; ++k) ms[k] = ctx->seg_ms[k];
    if (n) *n = SEG_N;
    return SPH_OK;
}

int sph_step_timed(sph_ctx *ctx, int n_steps, double *device_ms) {
    if (!ctx || !device_ms) return SPH_ERR_ARG;
    cudaSetDevice(ctx->device);
    SPH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    SPH_CUDA(ctx, cudaEventRecord(ctx->ev_begin, ctx->stream));
    SPH_TRY(sph_step(ctx, n_steps));
    SPH_CUDA(ctx, cudaEventRecord(ctx->ev_end, ctx->stream));
    SPH_CUDA(ctx, cudaEventSynchronize(ctx->ev_end));
    float ms = 0.0f;
    SPH_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev_begin, ctx->ev_end));
    *device_ms = ms;
    return SPH_OK;
}

int sph_get_counters(sph_ctx *ctx, int64_t out[16]) {
    if (!ctx || !out) return SPH_ERR_ARG;
    cudaSetDevice(ctx->device);
    int64_t w[8];
    SPH_TRY(sph_work_counts(ctx, w));
    out[8] = ctx->sup.rebuilds;
    out[9] = ctx->sup.repairs;
    out[10] = ctx->sup.violators;
    out[11] = ctx->sup.units_walked;
    out[12] = ctx->sup.n_units;
    out[13] = ctx->sup.K;
    out[14] = w[7];
    out[15] = ctx->sup.spill_on ? ctx->sup.spilled : 0;   // entries in spill ranges (rows longer than K)
    out[0] = ctx->launches;
    out[1] = w[0];
    out[2] = w[1];
    out[3] = w[2];
    out[4] = w[3];
    out[5] = w[4];
    out[6] = w[5];
    out[7] = w[6];
    return SPH_OK;
}

}  // extern "C"
