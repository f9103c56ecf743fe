// Mode 2 of the reference's step loop (main.cpp:155-158): SetConstantEntropy
// and CalcAll (force.h:55-84).  Per particle, after the final kick:
//   ent  = mantle_entropy for material 0 (the reference's tag 0), core_entropy otherwise
//   eng  = EoS::InternalEnergy(dens, ent)   RestrictedBilinearInterpolation, interpolation.h:107-335
//   temp = EoS::Temperature(dens, eng)      BilinearInterpolation on column 2, EoS.h:258-260, 411-413
//
// InternalEnergy in the reference finds two density slices of the table with
// linear scans over every table line (the "lower" one over a reversed copy of
// the line densities, made per call) and then the entries nearest to the
// entropy with a scan of each slice: O(lines) work per particle.  Here:
//  * the slice bounds come from two binary searches over the line densities,
//    which give the same lines as the scans because the table setter requires
//    the line densities to be non-decreasing;
//  * every particle of a material has the same entropy, so the energy at that
//    entropy on every possible slice is computed once per material
//    (k_entropy_edges, one thread per slice, the nearest-entropy scan kept
//    literal), leaving per particle two binary searches, two reads of that
//    table and one linear interpolation in density (k_entropy_step).
// All of it is FP64 in the reference's operation order with no fused
// multiply-adds, so the energies are bit-identical to a scalar evaluation.
// Where the reference would index outside its vectors (undefined behaviour
// there), the energy is NaN and the lookup is counted; sph_step then fails.
#include "sph_internal.cuh"
#include "sph_physics.cuh"

namespace sph {
namespace {

constexpr int ET = 256;

// get_neighbors_restricted_indices (interpolation.h:131-182) when its scan stops
// at line `hit` (-1: no line passes the test), in the reference's unsigned
// 32-bit index arithmetic.  Lower bound: hit = last line with density <= rho;
// upper bound: hit = first line with density >= rho.
__device__ void restricted_bounds(int64_t size, int64_t hit, uint32_t G, bool upper, uint32_t &b1, uint32_t &b2) {
    uint32_t lo = 0, hi = 0;
    if (hit >= 0) {
        if (upper) {
            lo = (uint32_t)hit;
            hi = (uint32_t)hit + G;
            if ((uint64_t)hi > (uint64_t)(size - 1)) hi = (uint32_t)(size - 1);
        } else {
            lo = (uint32_t)hit - (G - 1u);   // (size - 1) - a - (G - 1), a = size - 1 - hit
            hi = lo + G;
            if (hi == 0) hi = G;
        }
    }
    if (lo == 0 && hi == 0) {
        lo = 0;
        hi = G;
    }
    b1 = lo;
    b2 = hi;
}

// linear_interpolate (interpolation.h:254-262), rounded operation by operation
__device__ __forceinline__ double lerp_ref(double x1, double x2, double x, double q1, double q2) {
    const double d = __dsub_rn(x2, x1);
    return __dadd_rn(__dmul_rn(__ddiv_rn(__dsub_rn(x2, x), d), q1), __dmul_rn(__ddiv_rn(__dsub_rn(x, x1), d), q2));
}

// abs() of a double as the reference's translation unit resolves it: int
// abs(int) of the value truncated toward zero, defined for -2^31 < d < 2^31
__device__ __forceinline__ bool int_abs(double d, long long &out) {
    if (!(d > -2147483648.0 && d < 2147483648.0)) return false;
    const long long t = (long long)d;
    out = t < 0 ? -t : t;
    return true;
}

// The slice that a scan stopping at `hit` selects, and the energy at entropy
// s on it: get_var2_neighbors (interpolation.h:186-238) then the first
// linear_interpolate of interpolate_restricted (interpolation.h:240-252).
__device__ EntropyEdge entropy_edge(const DevMaterial &m, int64_t hit, bool upper, double s, uint32_t G,
                                    int abs_mode) {
    EntropyEdge e;
    e.p = e.u = __longlong_as_double(0x7ff8000000000000ll);
    e.undef = 1;
    e.pad = 0;
    const int64_t size = (int64_t)m.n_rho * m.n_u;
    uint32_t b1, b2;
    restricted_bounds(size, hit, G, upper, b1, b2);
    const int64_t lo = (int32_t)b1, hi = (int32_t)b2;   // slice(v, int m, int n), interpolation.h:17-25
    if (!(lo >= 0 && lo <= hi + 1 && hi + 1 <= size)) return e;
    const int64_t L = hi - lo + 1;
    const double *se = m.ent + lo;
    double min_d = 0.0;
    uint32_t idx = 0;
    bool ok = true;
    for (int64_t a = 0; a < L; ++a) {
        const double d = __dsub_rn(s, se[a]);
        if (a == 0) {
            min_d = d;
            continue;
        }
        bool closer;
        if (abs_mode == SPH_ENTROPY_ABS_INT) {
            long long di = 0, dm = 0;
            ok = int_abs(d, di) && ok;
            ok = int_abs(min_d, dm) && ok;
            closer = di < dm;
        } else {
            closer = fabs(d) < fabs(min_d);
        }
        if (closer) {
            min_d = d;
            idx = (uint32_t)a;
        }
    }
    uint32_t f, g;
    if (min_d < 0) {
        if (idx <= 0) { f = idx; g = idx + 1; }
        else if (idx + 1 == G) { f = idx - 2; g = idx - 1; }
        else { f = idx - 1; g = idx; }
    } else if (min_d > 0) {
        if (idx + 1 == G) { f = idx - 2; g = idx - 1; }
        else { f = idx; g = idx + 1; }
    } else {
        if (idx >= G - 1) { f = idx - 2; g = idx - 1; }
        else { f = idx - 1; g = idx + 1; }
    }
    const int64_t fi = (int32_t)f, gi = (int32_t)g;
    if (!ok || L < 1 || fi < 0 || gi < 0 || fi >= L || gi >= L) return e;
    e.p = m.line_rho[lo];
    e.u = lerp_ref(se[fi], se[gi], s, m.line_u[lo + fi], m.line_u[lo + gi]);
    e.undef = 0;
    return e;
}

// Where the reference's two scans stop: k = last line with density <= rho
// (-1: none), a = first line with density >= rho (-1: none).  Binary searches
// over the non-decreasing line densities; a NaN density passes no test.
__device__ __forceinline__ void line_hits(const double *v, int64_t size, double rho, int64_t &k, int64_t &a) {
    if (rho != rho) {
        k = -1;
        a = -1;
        return;
    }
    int64_t lo = 0, len = size;
    while (len > 0) {   // first line with rho < v
        const int64_t half = len >> 1;
        if (!(rho < v[lo + half])) {
            lo += half + 1;
            len -= half + 1;
        } else {
            len = half;
        }
    }
    k = lo - 1;
    lo = 0;
    len = size;
    while (len > 0) {   // first line with !(v < rho)
        const int64_t half = len >> 1;
        if (v[lo + half] < rho) {
            lo += half + 1;
            len -= half + 1;
        } else {
            len = half;
        }
    }
    a = lo < size ? lo : -1;
}

__device__ __forceinline__ double nan_d() { return __longlong_as_double(0x7ff8000000000000ll); }

// every slice of one material at its entropy: lo[k + 1] for the lower scan
// stopping at k in [-1, size), up[a] for the upper scan stopping at a in
// [0, size) and up[size] for "no line"
__global__ void k_entropy_edges(DevMaterial m, double s, uint32_t G, int abs_mode, EntropyEdge *lo, EntropyEdge *up) {
    const int64_t size = (int64_t)m.n_rho * m.n_u;
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t <= size) {
        lo[t] = entropy_edge(m, t - 1, false, s, G, abs_mode);
    } else if (t <= 2 * size + 1) {
        const int64_t a = t - size - 1;
        up[a] = entropy_edge(m, a < size ? a : -1, true, s, G, abs_mode);
    }
}

// SetConstantEntropy + CalcAll per particle (force.h:55-84).  A run whose
// step has dt 0 is taking its prologue (main.cpp:92-105, no CalcAll) and is
// left alone.
__global__ void __launch_bounds__(ET) k_entropy_step(int n, const DevMaterial *__restrict__ mats,
                                                     const int32_t *__restrict__ mat, const double *__restrict__ dens,
                                                     double *__restrict__ eng, double *__restrict__ ent,
                                                     double *__restrict__ temp, const int *__restrict__ prun,
                                                     const double *__restrict__ run_dt, double s_mantle,
                                                     double s_core, int *bad) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (run_dt[prun[i]] == 0.0) return;
    const int mi = mat[i];
    const DevMaterial &m = mats[mi];
    const double s = mi == 0 ? s_mantle : s_core;
    const double rho = dens[i];
    double u, T;
    bool fail = false;
    if (m.kind == 2) {   // IdealGas::InternalEnergy / Temperature return 0 (EoS.h:51-61)
        u = 0.0;
        T = 0.0;
    } else if (m.kind == 0 && m.edge_lo) {
        const int64_t size = (int64_t)m.n_rho * m.n_u;
        int64_t k, a;
        line_hits(m.line_rho, size, rho, k, a);
        const EntropyEdge el = m.edge_lo[k + 1], eu = m.edge_up[a < 0 ? size : a];
        fail = el.undef || eu.undef;
        u = fail ? nan_d() : lerp_ref(el.p, eu.p, rho, el.u, eu.u);
        T = table_lookup1(m, m.temp, rho, u);
    } else {
        fail = true;
        u = T = nan_d();
    }
    ent[i] = s;
    eng[i] = u;
    temp[i] = T;
    if (fail || !isfinite(u)) atomicAdd(bad, 1);
}

// sph_eos_eval: one EoS quantity at n points
__global__ void k_eos_points(int n, DevMaterial m, int quantity, const double *a, const double *b, double *out,
                             uint32_t G, int abs_mode, unsigned long long *undef) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double x = a[i], y = b[i];
    double v = nan_d();
    bool fail = false;
    if (quantity == SPH_EOS_PRESSURE || quantity == SPH_EOS_SOUND_SPEED) {
        double P, cs;
        eos_eval(m, x, y, P, cs);
        v = quantity == SPH_EOS_PRESSURE ? P : cs;
    } else if (m.kind == 2) {
        v = 0.0;
    } else if (m.kind != 0) {
        fail = true;
    } else if (quantity == SPH_EOS_TEMPERATURE || quantity == SPH_EOS_ENTROPY) {
        const double *plane = quantity == SPH_EOS_TEMPERATURE ? m.temp : m.ent;
        if (plane) v = table_lookup1(m, plane, x, y);
        else fail = true;
    } else if (m.ent && m.line_rho && m.line_u) {
        const int64_t size = (int64_t)m.n_rho * m.n_u;
        int64_t k, h;
        line_hits(m.line_rho, size, x, k, h);
        const EntropyEdge el = entropy_edge(m, k, false, y, G, abs_mode);
        const EntropyEdge eu = entropy_edge(m, h, true, y, G, abs_mode);
        fail = el.undef || eu.undef;
        if (!fail) v = lerp_ref(el.p, eu.p, x, el.u, eu.u);
    } else {
        fail = true;
    }
    out[i] = v;
    if (fail) atomicAdd(undef, 1ull);
}

int build_edges(sph_ctx *ctx) {
    const uint32_t G = (uint32_t)ctx->cfg.entropy_grid;
    for (int k = 0; k < MAX_MATERIALS; ++k) {
        DevMaterial &m = ctx->mats_host[k];
        if (ctx->m2_edges[k]) {
            SPH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            cudaFree(ctx->m2_edges[k]);
            ctx->m2_edges[k] = nullptr;
        }
        m.edge_lo = m.edge_up = nullptr;
        if (m.kind != 0 || !m.ent || !m.line_rho || !m.line_u) continue;
        const int64_t size = (int64_t)m.n_rho * m.n_u;
        EntropyEdge *e = nullptr;
        if (cudaMalloc((void **)&e, sizeof(EntropyEdge) * 2 * (size_t)(size + 1)) != cudaSuccess) {
            cudaGetLastError();
            return sph_fail(ctx, SPH_ERR_OOM, "mode-2 slices of material %d", k);
        }
        ctx->m2_edges[k] = e;
        const double s = k == 0 ? ctx->cfg.mantle_entropy : ctx->cfg.core_entropy;
        const int64_t threads = 2 * (size + 1);
        k_entropy_edges<<<sph_div_up(threads, ET), ET, 0, ctx->stream>>>(m, s, G, ctx->cfg.entropy_abs, e,
                                                                         e + size + 1);
        ++ctx->launches;
        SPH_CUDA(ctx, cudaGetLastError());
        m.edge_lo = e;
        m.edge_up = e + size + 1;
    }
    SPH_CUDA(ctx, cudaMemcpyAsync(ctx->mats_dev, ctx->mats_host, sizeof(ctx->mats_host), cudaMemcpyHostToDevice,
                                  ctx->stream));
    SPH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->m2_dirty = false;
    return SPH_OK;
}

}  // namespace
}  // namespace sph

using namespace sph;

int sph_entropy_step(sph_ctx *ctx) {
    if (ctx->m2_dirty) SPH_TRY(build_edges(ctx));
    if (!ctx->m2_bad) {
        if (cudaMalloc((void **)&ctx->m2_bad, sizeof(int)) != cudaSuccess) {
            cudaGetLastError();
            return sph_fail(ctx, SPH_ERR_OOM, "mode-2 counter");
        }
    }
    SPH_CUDA(ctx, cudaMemsetAsync(ctx->m2_bad, 0, sizeof(int), ctx->stream));
    const int n = (int)ctx->n;
    if (n == 0) return SPH_OK;
    double *F = ctx->F;
    const int64_t c = ctx->cap;
    k_entropy_step<<<sph_div_up(n, ET), ET, 0, ctx->stream>>>(
        n, ctx->mats_dev, ctx->mat, F + SPH_DENS * c, F + SPH_ENG * c, F + SPH_ENT * c, F + SPH_TEMP * c,
        ctx->runs.prun, ctx->runs.dt_dev, ctx->cfg.mantle_entropy, ctx->cfg.core_entropy, ctx->m2_bad);
    ++ctx->launches;
    SPH_CUDA(ctx, cudaGetLastError());
    return SPH_OK;
}

int sph_entropy_check(sph_ctx *ctx) {
    int bad = 0;
    SPH_CUDA(ctx, cudaMemcpyAsync(&bad, ctx->m2_bad, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    SPH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (bad)
        return sph_fail(ctx, SPH_ERR_NONFINITE,
                        "mode 2: %d particles have an InternalEnergy lookup that is undefined in the reference "
                        "(outside its table vectors) or not finite",
                        bad);
    return SPH_OK;
}

void sph_entropy_free(sph_ctx *ctx) {
    for (int k = 0; k < MAX_MATERIALS; ++k) {
        if (ctx->m2_edges[k]) cudaFree(ctx->m2_edges[k]);
        ctx->m2_edges[k] = nullptr;
    }
    if (ctx->m2_bad) cudaFree(ctx->m2_bad);
    ctx->m2_bad = nullptr;
}

extern "C" int sph_eos_eval(sph_ctx *ctx, int material, int quantity, int64_t n, const double *a, const double *b,
                            double *out, int64_t *undefined) {
    if (!ctx) return SPH_ERR_ARG;
    if (material < 0 || material >= MAX_MATERIALS) return sph_fail(ctx, SPH_ERR_ARG, "material %d out of range", material);
    if (quantity < SPH_EOS_PRESSURE || quantity > SPH_EOS_INTERNAL_ENERGY)
        return sph_fail(ctx, SPH_ERR_ARG, "unknown EoS quantity %d", quantity);
    if (n < 0 || n > (int64_t)1 << 30 || (n > 0 && (!a || !b || !out))) return sph_fail(ctx, SPH_ERR_ARG, "bad points");
    if (undefined) *undefined = 0;
    if (n == 0) return SPH_OK;
    cudaSetDevice(ctx->device);
    const DevMaterial &m = ctx->mats_host[material];
    if (m.kind < 0) return sph_fail(ctx, SPH_ERR_TABLE, "material %d is not set", material);
    double *d = nullptr;
    unsigned long long *cnt = nullptr;
    if (cudaMalloc((void **)&d, sizeof(double) * 3 * (size_t)n) != cudaSuccess ||
        cudaMalloc((void **)&cnt, sizeof(unsigned long long)) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(d);
        return sph_fail(ctx, SPH_ERR_OOM, "EoS evaluation buffers");
    }
    int rc = SPH_OK;
    unsigned long long bad = 0;
    do {
        if (cudaMemcpyAsync(d, a, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess ||
            cudaMemcpyAsync(d + n, b, sizeof(double) * n, cudaMemcpyHostToDevice, ctx->stream) != cudaSuccess ||
            cudaMemsetAsync(cnt, 0, sizeof(unsigned long long), ctx->stream) != cudaSuccess) {
            rc = sph_fail(ctx, SPH_ERR_CUDA, "EoS evaluation copies");
            break;
        }
        k_eos_points<<<sph_div_up(n, ET), ET, 0, ctx->stream>>>((int)n, m, quantity, d, d + n, d + 2 * n,
                                                                (uint32_t)ctx->cfg.entropy_grid, ctx->cfg.entropy_abs,
                                                                cnt);
        ++ctx->launches;
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpyAsync(out, d + 2 * n, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
            cudaMemcpyAsync(&bad, cnt, sizeof(bad), cudaMemcpyDeviceToHost, ctx->stream) != cudaSuccess ||
            cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
            rc = sph_fail(ctx, SPH_ERR_CUDA, "EoS evaluation kernel");
            break;
        }
    } while (false);
    cudaFree(d);
    cudaFree(cnt);
    if (rc == SPH_OK && undefined) *undefined = (int64_t)bad;
    return rc;
}
