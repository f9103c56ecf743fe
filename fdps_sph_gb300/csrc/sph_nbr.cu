// SPH neighbour lists: one tree walk per step, exact lists per pass.
//
// The reference gets an i-group and a superset j-list from FDPS for every
// density, derivative and hydro call (TreeForForceShort::Gather / Symmetry,
// main.cpp:79-81, 139-143).  Here the j-sets are explicit: for particle i
//   gather    : { j : |x_j - x_i|^2 < (2.5 h_i)^2 }            (density, derivative)
//   symmetric : { j : |x_j - x_i|^2 < max(2.5 h_i, 2.5 h_j)^2 }  (hydro)
// in ascending key order, identical to the oracle's (oracle/sph_oracle.c:
// or_sph_walk).
//
// 1. Units: octree cells with at most 32 particles whose parent holds more;
//    consecutive sibling units are packed into one warp while they fit.
//    Units are spatially compact (inside one parent cell), so no warp sees
//    a group box that straddles a jump of the Morton curve.
// 2. Superset walk, once per step (after the sort): every warp walks the
//    octree depth-first in octant order with its unit's bounding box and
//    keeps j with r_ij < KAPPA * max(H_i, H_j) (FP32 with a generous margin),
//    the h of that moment being recorded as h_sup.
// 3. Per pass, a filter kernel keeps the exact set from the superset: FP32
//    on double-float coordinates with an error band of 2^-19 relative, the
//    exact FP64 test of the oracle inside the band.  The superset contains
//    the exact set as long as every h <= KAPPA * h_sup; the filter raises a
//    flag otherwise and the host rebuilds the superset with the current h.
#include <algorithm>
#include <cstring>

#include "sph_fixpoint.cuh"
#include "sph_internal.cuh"

namespace sph {

constexpr int UNIT = 32;
constexpr float KAPPA = 1.06f;   // measured at 1M: 1.15 -> 13.7 ms, 1.10 -> 12.9, 1.06 -> 12.6, 1.03 -> 13.0 (repairs)
// walk warps per block: one, so a block's SM slot is freed as soon as its walk unit is done (the
// units' walks differ in length); 1M walk: 1.95 ms with four warps per block, 1.97 with two,
// 1.92 with one (about 30 blocks per SM, limited by shared memory)
constexpr int NB_WARPS = 1;
constexpr int ROW_K_MAX = 512;   // widest row block; longer rows continue in spill ranges (RowMap)
constexpr int NB_CAND = 256;   // raw candidate indices per warp (flushes half as often as with 128: -0.02 ms at 1M)
constexpr int NB_SURV = 64;    // culled candidates staged for the pair test
constexpr int NB_STACK = 264;   // depth-first from any stack of <= NB_MULTI entries: + 21 levels x 7 pending siblings + 1
constexpr int NB_MULTI = 116;   // the stack may reach this with several cells expanded at once
constexpr unsigned FULLM = 0xffffffffu;

__device__ __forceinline__ float df_sub(float ah, float al, float bh, float bl) { return (ah - bh) + (al - bl); }

// ---------------------------------------------------------------------------
// units

// number of units contributed by cell c (see file comment); EMIT writes them at off[c]
template <bool EMIT>
__global__ void k_units(const int *meta, const int *start, const int *count, const int *first_child,
                        const int *n_child, int *nunits, const int *off, int2 *units) {
    const int nc = meta[MAX_LEVELS], n_roots = meta[1];
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        const int cnt = count[c], nch = n_child[c];
        const bool root = c < n_roots;   // level 0: one root per run
        int k = 0;
        int2 *out = EMIT ? units + off[c] : nullptr;
        if (root && cnt <= UNIT) {
            if (EMIT) out[k] = make_int2(start[c], cnt);
            ++k;
        } else if (root && nch == 0) {
            for (int s = 0; s < cnt; s += UNIT) {
                if (EMIT) out[k] = make_int2(start[c] + s, min(UNIT, cnt - s));
                ++k;
            }
        } else if (cnt > UNIT && nch > 0) {
            const int f = first_child[c];
            int us = -1, un = 0;
            for (int q = 0; q < nch; ++q) {
                const int ch = f + q, cc = count[ch];
                if (cc <= UNIT) {
                    if (us >= 0 && un + cc <= UNIT) {
                        un += cc;
                    } else {
                        if (us >= 0) {
                            if (EMIT) out[k] = make_int2(us, un);
                            ++k;
                        }
                        us = start[ch];
                        un = cc;
                    }
                } else {
                    if (us >= 0) {
                        if (EMIT) out[k] = make_int2(us, un);
                        ++k;
                    }
                    us = -1;
                    un = 0;
                    if (n_child[ch] == 0) {   // a leaf above the unit size (only at the deepest level)
                        for (int s = 0; s < cc; s += UNIT) {
                            if (EMIT) out[k] = make_int2(start[ch] + s, min(UNIT, cc - s));
                            ++k;
                        }
                    }
                }
            }
            if (us >= 0) {
                if (EMIT) out[k] = make_int2(us, un);
                ++k;
            }
        }
        if (!EMIT) nunits[c] = k;
    }
}

// ---------------------------------------------------------------------------
// superset walk: one warp per unit

struct WalkTree {
    const int4 *cinfo;   // first_child, n_child, start, count
    const float4 *blo, *bhi;
};

__device__ __forceinline__ float gap2_rd(float4 a_lo, float4 a_hi, float3 glo, float3 ghi) {
    const float gx = fmaxf(0.0f, fmaxf(__fsub_rd(a_lo.x, ghi.x), __fsub_rd(glo.x, a_hi.x)));
    const float gy = fmaxf(0.0f, fmaxf(__fsub_rd(a_lo.y, ghi.y), __fsub_rd(glo.y, a_hi.y)));
    const float gz = fmaxf(0.0f, fmaxf(__fsub_rd(a_lo.z, ghi.z), __fsub_rd(glo.z, a_hi.z)));
    return __fadd_rd(__fadd_rd(__fmul_rd(gx, gx), __fmul_rd(gy, gy)), __fmul_rd(gz, gz));
}

// SPILL: rows may continue in spill ranges (walks after this step's spill layout); without it
// the hot loop carries no spill code (a row longer than K only raises the overflow flag)
template <bool SPILL>
__global__ void __launch_bounds__(NB_WARPS * 32, 32 / NB_WARPS)
k_sup_walk(int n_units, const int2 *__restrict__ units, const int *__restrict__ uidx, const double *__restrict__ x,
           const double *__restrict__ y, const double *__restrict__ z, const double *__restrict__ h,
           double *__restrict__ hsup, const float4 *__restrict__ xh,
           const float4 *__restrict__ xl, const float *__restrict__ H2f, const int *__restrict__ prun, WalkTree T,
           int *__restrict__ sup,
           float *__restrict__ sup_r2, float *__restrict__ sup_m, int *__restrict__ cnt, RowMap rm, int *uover,
           int *err, int *maxcnt) {
    // cells to visit: (first_child, -n_child) for an internal cell, (start, count) for a leaf
    __shared__ int2 s_stack[NB_WARPS][NB_STACK];
    __shared__ int s_cand[NB_WARPS][NB_CAND];
    // candidates that survived the per-particle cull: index, hi, lo (.w = (2.5 h_j)^2 rounded up)
    __shared__ int s_sj[NB_WARPS][NB_SURV];
    __shared__ float4 s_ph[NB_WARPS][NB_SURV];
    __shared__ float4 s_pl[NB_WARPS][NB_SURV];
    // every lane's double-float position, for the lanes that write another lane's entries
    __shared__ float4 s_pih[NB_WARPS][32], s_pil[NB_WARPS][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int w = blockIdx.x * NB_WARPS + warp;
    if (w >= n_units) return;   // warp-uniform
    const int uid = uidx ? uidx[w] : w;
    const int2 U = units[uid];
    const int K = rm.K;
    const bool valid = lane < U.y;
    const int i = U.x + (valid ? lane : 0);
    const double xi = x[i], yi = y[i], zi = z[i];
    if (valid) hsup[i] = h[i];   // the h this row is built for
    const float4 pih = xh[i], pil = xl[i];
    const float H2i = valid ? H2f[i] : 0.0f;
    double lo[3] = {valid ? xi : INFINITY, valid ? yi : INFINITY, valid ? zi : INFINITY};
    double hi[3] = {valid ? xi : -INFINITY, valid ? yi : -INFINITY, valid ? zi : -INFINITY};
    float R2 = H2i;
    for (int o = 16; o > 0; o >>= 1) {
        for (int d = 0; d < 3; ++d) {
            lo[d] = fmin(lo[d], __shfl_xor_sync(FULLM, lo[d], o));
            hi[d] = fmax(hi[d], __shfl_xor_sync(FULLM, hi[d], o));
        }
        R2 = fmaxf(R2, __shfl_xor_sync(FULLM, R2, o));
    }
    const float3 glo = make_float3(__double2float_rd(lo[0]), __double2float_rd(lo[1]), __double2float_rd(lo[2]));
    const float3 ghi = make_float3(__double2float_ru(hi[0]), __double2float_ru(hi[1]), __double2float_ru(hi[2]));
    const float k2 = KAPPA * KAPPA * 1.00390625f;          // kappa^2 (1 + 2^-8): generous, only a superset is needed
    const float Rg = __fmul_ru(KAPPA * 1.00390625f, __fsqrt_ru(R2));
    const float Rg2 = __fmul_ru(Rg, Rg);
    const unsigned lt = (1u << lane) - 1u;
    int2 *stack = s_stack[warp];
    int *cand = s_cand[warp];
    int count = 0, nc = 0;
    // the spill range continues a row at entry K: entry k >= K of particle p at
    // rm.main + rm.soff[p] - K + k (computed on the rare paths that need it)
    auto spill_cap = [&]() { return valid ? row_spill_cap(rm, i) : 0; };
    s_pih[warp][lane] = pih;
    s_pil[warp][lane] = pil;
    __syncwarp();

    // Candidates are culled 32 at a time, each against the unit's box grown by its own reach:
    // a lower bound of the distance (the point's hi / lo interval, rounded down) against an
    // upper bound of max(Rg, kappa' 2.5 h_j), so no pair the test below would accept is
    // dropped.  Survivors are staged with their coordinates and tested against every lane.
    auto flush = [&]() {
        int ns = 0;
        for (int b = 0; b < nc; b += 32) {
            const int kk = b + lane;
            bool keep = false;
            int j = 0;
            float4 qh = make_float4(0.f, 0.f, 0.f, 0.f), ql = qh;
            if (kk < nc) {
                j = cand[kk];
                qh = xh[j];
                ql = xl[j];
                ql.w = H2f[j];
                const float ex = fabsf(ql.x), ey = fabsf(ql.y), ez = fabsf(ql.z);
                const float gx = fmaxf(0.0f, fmaxf(__fsub_rd(__fsub_rd(qh.x, ex), ghi.x),
                                                   __fsub_rd(glo.x, __fadd_ru(qh.x, ex))));
                const float gy = fmaxf(0.0f, fmaxf(__fsub_rd(__fsub_rd(qh.y, ey), ghi.y),
                                                   __fsub_rd(glo.y, __fadd_ru(qh.y, ey))));
                const float gz = fmaxf(0.0f, fmaxf(__fsub_rd(__fsub_rd(qh.z, ez), ghi.z),
                                                   __fsub_rd(glo.z, __fadd_ru(qh.z, ez))));
                const float g2 = __fadd_rd(__fadd_rd(__fmul_rd(gx, gx), __fmul_rd(gy, gy)), __fmul_rd(gz, gz));
                keep = g2 < fmaxf(Rg2, __fmul_ru(k2, ql.w));
            }
            const unsigned km = __ballot_sync(FULLM, keep);
            if (keep) {
                const int p = ns + __popc(km & lt);
                s_sj[warp][p] = j;
                s_ph[warp][p] = qh;
                s_pl[warp][p] = ql;
            }
            ns += __popc(km);
            __syncwarp();
            if (ns >= 32 || b + 32 >= nc) {
                // every lane tests every survivor without branching (bit t of `am`), then writes
                // its accepted ones in survivor order; the warp diverges only over those
                unsigned amw[2] = {0u, 0u};
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int t1 = min(ns, 32 * h + 32);
#pragma unroll 4
                    for (int t = 32 * h; t < t1; ++t) {
                        const float4 ph = s_ph[warp][t], pl = s_pl[warp][t];
                        const float dx = df_sub(ph.x, pl.x, pih.x, pil.x);
                        const float dy = df_sub(ph.y, pl.y, pih.y, pil.y);
                        const float dz = df_sub(ph.z, pl.z, pih.z, pil.z);
                        const float r2 = dx * dx + dy * dy + dz * dz;
                        amw[h] |= (unsigned)(r2 < k2 * fmaxf(H2i, pl.w)) << (t - 32 * h);
                    }
                }
                unsigned long long am = ((unsigned long long)amw[1] << 32) | amw[0];
                if (!valid) am = 0ull;
                // The batch's accepted entries, lane by lane and in survivor order within a lane,
                // are numbered e = 0 .. total - 1 and written by the whole warp, 32 at a time: a
                // lane's run of entries lands contiguously in its row, so every store covers a few
                // runs instead of 32 rows.  Entry e belongs to lane L (prefix[L] <= e < prefix[L]
                // + nacc[L]) and is that lane's k-th accepted survivor, k = e - prefix[L].
                const unsigned alo = (unsigned)am, ahi = (unsigned)(am >> 32);
                const int nacc = __popc(alo) + __popc(ahi);
                int incl = nacc;
                for (int o = 1; o < 32; o <<= 1) {
                    const int v = __shfl_up_sync(FULLM, incl, o);
                    if (lane >= o) incl += v;
                }
                const int total = __shfl_sync(FULLM, incl, 31);
                for (int e0 = 0; e0 < total; e0 += 32) {
                    const int e = e0 + lane;
                    int L = 0;   // the owner: the number of lanes whose inclusive prefix is <= e
                    for (int st = 16; st > 0; st >>= 1) {
                        const int v = __shfl_sync(FULLM, incl, L + st - 1);
                        if (v <= e) L += st;
                    }
                    L = min(L, 31);
                    const int excl = __shfl_sync(FULLM, incl - nacc, L);
                    const unsigned lo = __shfl_sync(FULLM, alo, L), hi = __shfl_sync(FULLM, ahi, L);
                    const int base = __shfl_sync(FULLM, count, L);
                    if (e < total) {
                        // t = the position of the k-th set bit of the 64-bit mask hi:lo, by halving with
                        // popc (__fns here cost 0.17 ms of the walk's 2.55 ms per 1M step)
                        const int k = e - excl;
                        int kk = k, t = 0;
                        unsigned x = lo;
                        const int plo = __popc(lo);
                        if (kk >= plo) {
                            kk -= plo;
                            x = hi;
                            t = 32;
                        }
#pragma unroll
                        for (int w = 16; w >= 1; w >>= 1) {
                            const int c = __popc(x & ((1u << w) - 1u));
                            if (kk >= c) {
                                kk -= c;
                                x >>= w;
                                t += w;
                            }
                        }
                        const float4 ph = s_ph[warp][t], pl = s_pl[warp][t];
                        const float4 qh = s_pih[warp][L], ql = s_pil[warp][L];
                        const float dx = df_sub(ph.x, pl.x, qh.x, ql.x);
                        const float dy = df_sub(ph.y, pl.y, qh.y, ql.y);
                        const float dz = df_sub(ph.z, pl.z, qh.z, ql.z);
                        const float r2 = dx * dx + dy * dy + dz * dz;
                        const int iL = U.x + L, pos = base + k;
                        if (pos < K) {
                            const int64_t o = (int64_t)iL * K + pos;
                            sup[o] = s_sj[warp][t];
                            sup_r2[o] = r2;
                            sup_m[o] = ph.w;
                        } else if (SPILL && pos < K + row_spill_cap(rm, iL)) {
                            const int64_t o = rm.main + rm.soff[iL] - K + pos;
                            sup[o] = s_sj[warp][t];
                            sup_r2[o] = r2;
                            sup_m[o] = ph.w;
                        }
                    }
                }
                count += nacc;
                ns = 0;
                __syncwarp();
            }
        }
        nc = 0;
    };

    int sp = 0;
    {
        const int root = prun[U.x];   // the unit's run's octree root
        const float4 a = T.blo[root], b = T.bhi[root];
        const float R = fmaxf(Rg, __fmul_ru(2.5f * KAPPA * 1.00390625f, b.w));
        if (gap2_rd(a, b, glo, ghi) < __fmul_ru(R, R)) {
            if (lane == 0) {
                const int4 r = T.cinfo[root];
                stack[0] = r.y == 0 ? make_int2(r.z, r.w) : make_int2(r.x, -r.y);
            }
            sp = 1;
        }
        __syncwarp();
    }
    while (sp > 0) {
        const int2 ci = stack[sp - 1];
        if (ci.y > 0) {   // a leaf: with the leaves right below it, while their particles fit 32 lanes
            if (nc + 32 > NB_CAND) flush();
            int k = 1, tot = ci.y;
            while (k < 8 && sp - 1 - k >= 0) {
                const int2 nx = stack[sp - 1 - k];
                if (nx.y <= 0 || tot + nx.y > 32) break;
                tot += nx.y;
                ++k;
            }
            if (tot <= 32) {
                // lane -> (leaf, offset): leaves in stack order from the top, particles in order
                int acc = 0, src = -1;
                for (int g = 0; g < k; ++g) {
                    const int2 lf = stack[sp - 1 - g];
                    if (src < 0 && lane < acc + lf.y) src = lf.x + (lane - acc);
                    acc += lf.y;
                }
                __syncwarp();
                if (lane < tot) cand[nc + lane] = src;
                nc += tot;
                sp -= k;
                __syncwarp();
            } else {   // a leaf above 32 particles (only at the deepest level)
                --sp;
                __syncwarp();
                const int s = ci.x, ct = ci.y;
                for (int b0 = 0; b0 < ct; b0 += 32) {
                    if (nc + 32 > NB_CAND) flush();
                    if (b0 + lane < ct) cand[nc + lane] = s + b0 + lane;
                    nc += min(32, ct - b0);
                    __syncwarp();
                }
            }
        } else {
            // up to four internal cells from the top of the stack expanded at once, eight lanes per
            // cell: their children are pushed so that the top cell's come first, as the one-cell
            // expansion would visit them (the leaves, and so the rows, keep their order).  More
            // than one only while the stack stays below NB_MULTI, so a depth-first continuation
            // (at most 7 pending siblings per level below) still fits NB_STACK.
            int k = 1;
            while (k < 4 && sp - 1 - k >= 0 && stack[sp - 1 - k].y <= 0 && sp - (k + 1) + 8 * (k + 1) <= NB_MULTI) ++k;
            const int g = lane >> 3, q = lane & 7;
            bool ok = false;
            int2 chi = make_int2(0, 0);
            if (g < k) {
                const int2 cg = stack[sp - 1 - g];
                const int f = cg.x, nch = -cg.y;
                if (q < nch) {
                    const float4 a = T.blo[f + q], b = T.bhi[f + q];
                    const int4 r = T.cinfo[f + q];   // independent of the box loads: one round trip
                    chi = r.y == 0 ? make_int2(r.z, r.w) : make_int2(r.x, -r.y);
                    const float R = fmaxf(Rg, __fmul_ru(2.5f * KAPPA * 1.00390625f, b.w));
                    ok = gap2_rd(a, b, glo, ghi) < __fmul_ru(R, R);
                }
            }
            sp -= k;
            __syncwarp();
            const unsigned mask = __ballot_sync(FULLM, ok);
            const int np = __popc(mask);
            if (sp + np > NB_STACK) {
                if (lane == 0) atomicOr(err, ERR_SPH_STACK);
                break;
            }
            if (ok) stack[sp + (np - 1 - __popc(mask & ((1u << lane) - 1u)))] = chi;
            sp += np;
            __syncwarp();
        }
    }
    flush();
    if (valid) {
        const int scap = (SPILL && count > K) ? spill_cap() : 0;
        cnt[i] = count;   // the true count, also when the row had no room for all of it
        if (count > K + scap) atomicOr(err, ERR_SPH_LIST_OVERFLOW);
    }
    int m = valid ? count : 0;
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(FULLM, m, o));
    if (lane == 0) {
        atomicMax(maxcnt, m);
        uover[uid] = m > K ? 1 : 0;   // the unit holds rows that need a spill range
    }
}

// ---------------------------------------------------------------------------
// incremental repair after h outgrew the skin
//
// A row built when particle j had smoothing length h_j(T) keeps every
// neighbour as long as 2.5 h_j <= KAPPA * 2.5 h_j(T) for all j near it.  A
// particle v that violates this (h_v > KAPPA * hsup_v) can be missing from
// its own row and from the symmetric rows of particles within 2.5 h_v of it;
// the rows of every unit within reach of a violator are walked again.

__global__ void k_viol_mark(int n, const double *h, const double *hsup, float *vR, int *nviol) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    bool v = false;
    if (i < n) {
        v = h[i] > (double)KAPPA * hsup[i];
        vR[i] = v ? __double2float_ru(SUPPORT * h[i] * 1.001) : 0.0f;
    }
    const unsigned b = __ballot_sync(FULLM, v);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(nviol, __popc(b));
}

__global__ void k_cell_vmax(int l, const int *meta, const float *vR, const int4 *cinfo, float *cvR) {
    const int L0 = meta[l], L1 = meta[l + 1];
    for (int c = L0 + blockIdx.x * blockDim.x + threadIdx.x; c < L1; c += gridDim.x * blockDim.x) {
        const int4 ci = cinfo[c];
        float r = 0.0f;
        if (ci.y == 0) {
            for (int j = ci.z; j < ci.z + ci.w; ++j) r = fmaxf(r, vR[j]);
        } else {
            for (int k = 0; k < ci.y; ++k) r = fmaxf(r, cvR[ci.x + k]);
        }
        cvR[c] = r;
    }
}

// warp per unit: is any violator within its reach of the unit's box?
__global__ void __launch_bounds__(NB_WARPS * 32)
k_unit_mark(int n_units, const int2 *__restrict__ units, const float4 *__restrict__ xh, const float4 *__restrict__ xl,
            const float *__restrict__ vR, const float *__restrict__ cvR, const int4 *__restrict__ cinfo,
            const float4 *__restrict__ blo, const float4 *__restrict__ bhi, const int *__restrict__ prun,
            int *umark) {
    __shared__ int s_stack[NB_WARPS][NB_STACK];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int u = blockIdx.x * NB_WARPS + warp;
    if (u >= n_units) return;
    const int2 U = units[u];
    const bool valid = lane < U.y;
    const int i = U.x + (valid ? lane : 0);
    const float4 ph = xh[i], pl = xl[i];
    // unit box in float, widened by one ulp each way (the double-float sum rounds)
    float lo[3] = {valid ? ph.x + pl.x : INFINITY, valid ? ph.y + pl.y : INFINITY, valid ? ph.z + pl.z : INFINITY};
    float hi[3] = {valid ? ph.x + pl.x : -INFINITY, valid ? ph.y + pl.y : -INFINITY,
                   valid ? ph.z + pl.z : -INFINITY};
    for (int o = 16; o > 0; o >>= 1)
        for (int d = 0; d < 3; ++d) {
            lo[d] = fminf(lo[d], __shfl_xor_sync(FULLM, lo[d], o));
            hi[d] = fmaxf(hi[d], __shfl_xor_sync(FULLM, hi[d], o));
        }
    const float3 glo = make_float3(nextafterf(lo[0], -INFINITY), nextafterf(lo[1], -INFINITY),
                                   nextafterf(lo[2], -INFINITY));
    const float3 ghi = make_float3(nextafterf(hi[0], INFINITY), nextafterf(hi[1], INFINITY),
                                   nextafterf(hi[2], INFINITY));
    int *stack = s_stack[warp];
    int sp = 0;
    bool hit = false;
    {
        const int root = prun[U.x];   // the unit's run's octree root
        const float r = cvR[root];
        if (r > 0.0f && gap2_rd(blo[root], bhi[root], glo, ghi) < __fmul_ru(r, r)) {
            if (lane == 0) stack[0] = root;
            sp = 1;
        }
        __syncwarp();
    }
    while (sp > 0 && !hit) {
        const int c = stack[--sp];
        __syncwarp();
        const int4 ci = cinfo[c];
        if (ci.y == 0) {
            bool h2 = false;
            for (int j = ci.z + lane; j < ci.z + ci.w; j += 32) {
                const float r = vR[j];
                if (r > 0.0f) {
                    const float4 qh = xh[j], ql = xl[j];
                    const float px = qh.x + ql.x, py = qh.y + ql.y, pz = qh.z + ql.z;
                    const float4 a = make_float4(nextafterf(px, -INFINITY), nextafterf(py, -INFINITY),
                                                 nextafterf(pz, -INFINITY), 0.0f);
                    const float4 b = make_float4(nextafterf(px, INFINITY), nextafterf(py, INFINITY),
                                                 nextafterf(pz, INFINITY), 0.0f);
                    if (gap2_rd(a, b, glo, ghi) < __fmul_ru(r, r)) h2 = true;
                }
            }
            hit = __any_sync(FULLM, h2);
        } else {
            bool ok = false;
            int ch = 0;
            if (lane < ci.y) {
                ch = ci.x + lane;
                const float r = cvR[ch];
                ok = r > 0.0f && gap2_rd(blo[ch], bhi[ch], glo, ghi) < __fmul_ru(r, r);
            }
            const unsigned mask = __ballot_sync(FULLM, ok);
            const int np = __popc(mask);
            if (sp + np > NB_STACK) {   // cannot happen for an octree of depth 21; be safe: mark
                hit = true;
                break;
            }
            if (ok) stack[sp + (np - 1 - __popc(mask & ((1u << lane) - 1u)))] = ch;
            sp += np;
            __syncwarp();
        }
    }
    if (lane == 0) umark[u] = hit ? 1 : 0;
}

__global__ void k_unit_compact(int n_units, const int *umark, const int *off, int *uidx) {
    for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < n_units; u += gridDim.x * blockDim.x)
        if (umark[u]) uidx[off[u]] = u;
}

// ---------------------------------------------------------------------------
// exact filter: one thread per particle

constexpr int ERR_SKIN = 16;

// The FP32 r^2 stored by the walk is (x_j - x_i)^2 on double-float
// coordinates, within 2^-21 of the exact value; outside a band of 2^-19
// around the threshold it decides alone, inside it the oracle's FP64 test
// decides.
__device__ __forceinline__ bool exact_in(float r2, float thr, int j, double xi, double yi, double zi, double H2,
                                         const double *__restrict__ x, const double *__restrict__ y,
                                         const double *__restrict__ z, const double *__restrict__ h, bool sym) {
    if (r2 < thr * (1.0f - 1.9073486328125e-06f)) return true;
    if (r2 > thr * (1.0f + 1.9073486328125e-06f)) return false;
    const double ex = __dsub_rn(x[j], xi), ey = __dsub_rn(y[j], yi), ez = __dsub_rn(z[j], zi);
    const double rr = __dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez));
    if (rr < H2) return true;
    if (sym) {
        const double Hj = __dmul_rn(SUPPORT, h[j]);
        return rr < __dmul_rn(Hj, Hj);
    }
    return false;
}

// exact_in behind a call: a loop that decides several entries before summing them would
// otherwise have the FP64 test if-converted, issuing its FP64 instructions for every entry
__device__ __noinline__ bool exact_in_call(float r2, float thr, int j, double xi, double yi, double zi, double H2,
                                           const double *__restrict__ x, const double *__restrict__ y,
                                           const double *__restrict__ z, const double *__restrict__ h) {
    return exact_in(r2, thr, j, xi, yi, zi, H2, x, y, z, h, false);
}

template <int MODE>
__global__ void __launch_bounds__(128)
k_filter(int n, const int *__restrict__ sup, const float *__restrict__ sup_r2, const int *__restrict__ scnt,
         RowMap rm, const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ z,
         const double *__restrict__ h, const double *__restrict__ hsup, const float *__restrict__ H2f,
         int *__restrict__ out, int *__restrict__ ocnt, int *err) {
    __shared__ int s_buf[8][128];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double hi = h[i];
    const double Hi = __dmul_rn(SUPPORT, hi);
    const double H2 = __dmul_rn(Hi, Hi);
    const float H2i = (float)H2;
    const double xi = x[i], yi = y[i], zi = z[i];
    const int c = scnt[i];
    const int K = rm.K;
    int *orow = out + (int64_t)i * K;
    // the exact list is a subset of the superset row: it fits the row and the same spill range
    int *ospill = (c > K && rm.soff) ? out + rm.main + rm.soff[i] - K : nullptr;   // entry k >= K at ospill + k
    const int t = threadIdx.x;
    int k2 = 0;
    for (int seg = 0; seg < 2; ++seg) {
        int cs;
        const int64_t b = row_seg(rm, i, seg, c, &cs);
        if (cs <= 0) break;
        const int *row = sup + b;
        const float *rrow = sup_r2 + b;
        for (int k = 0; k < cs; k += 8) {
            const int4 j0 = reinterpret_cast<const int4 *>(row + k)[0], j1 = reinterpret_cast<const int4 *>(row + k)[1];
            const float4 r0 = reinterpret_cast<const float4 *>(rrow + k)[0],
                         r1 = reinterpret_cast<const float4 *>(rrow + k)[1];
            const int jj[8] = {j0.x, j0.y, j0.z, j0.w, j1.x, j1.y, j1.z, j1.w};
            const float rr[8] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w};
            const int m = min(8, cs - k);
            float thr[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) thr[u] = (MODE == 1 && u < m) ? fmaxf(H2i, H2f[jj[u]]) : H2i;
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                if (u < m && exact_in(rr[u], thr[u], jj[u], xi, yi, zi, H2, x, y, z, h, MODE == 1)) {
                    s_buf[k2 & 7][t] = jj[u];
                    ++k2;
                    if ((k2 & 7) == 0) {
                        int4 *dst = reinterpret_cast<int4 *>((k2 - 8 < K ? orow : ospill) + k2 - 8);
                        dst[0] = make_int4(s_buf[0][t], s_buf[1][t], s_buf[2][t], s_buf[3][t]);
                        dst[1] = make_int4(s_buf[4][t], s_buf[5][t], s_buf[6][t], s_buf[7][t]);
                    }
                }
            }
        }
    }
    for (int q = 0; q < (k2 & 7); ++q) {
        const int k = (k2 & ~7) + q;
        (k < K ? orow : ospill)[k] = s_buf[q][t];
    }
    ocnt[i] = k2;
}

// Both exact lists in one pass over the superset (the gather set is a subset of the symmetric
// set, so the gather test runs only on symmetric members); same decisions and order as
// k_filter<0> and k_filter<1>.
__global__ void __launch_bounds__(128)
k_filter2(int n, const int *__restrict__ sup, const float *__restrict__ sup_r2, const int *__restrict__ scnt,
          RowMap rm, const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ z,
          const double *__restrict__ h, const float *__restrict__ H2f, int *__restrict__ out0,
          int *__restrict__ ocnt0, int *__restrict__ out1, int *__restrict__ ocnt1) {
    __shared__ int s_b0[8][128], s_b1[8][128];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double hi = h[i];
    const double Hi = __dmul_rn(SUPPORT, hi);
    const double H2 = __dmul_rn(Hi, Hi);
    const float H2i = (float)H2;
    const double xi = x[i], yi = y[i], zi = z[i];
    const int c = scnt[i];
    const int K = rm.K;
    int *orow0 = out0 + (int64_t)i * K, *orow1 = out1 + (int64_t)i * K;
    const bool sp = c > K && rm.soff;
    int *osp0 = sp ? out0 + rm.main + rm.soff[i] - K : nullptr, *osp1 = sp ? out1 + rm.main + rm.soff[i] - K : nullptr;
    const int t = threadIdx.x;
    int k0 = 0, k1 = 0;
    auto put = [&](int (*buf)[128], int &kk, int *orow, int *osp, int j) {
        buf[kk & 7][t] = j;
        ++kk;
        if ((kk & 7) == 0) {
            int4 *dst = reinterpret_cast<int4 *>((kk - 8 < K ? orow : osp) + kk - 8);
            dst[0] = make_int4(buf[0][t], buf[1][t], buf[2][t], buf[3][t]);
            dst[1] = make_int4(buf[4][t], buf[5][t], buf[6][t], buf[7][t]);
        }
    };
    for (int seg = 0; seg < 2; ++seg) {
        int cs;
        const int64_t b = row_seg(rm, i, seg, c, &cs);
        if (cs <= 0) break;
        const int *row = sup + b;
        const float *rrow = sup_r2 + b;
        for (int k = 0; k < cs; k += 8) {
            const int4 j0 = reinterpret_cast<const int4 *>(row + k)[0], j1 = reinterpret_cast<const int4 *>(row + k)[1];
            const float4 r0 = reinterpret_cast<const float4 *>(rrow + k)[0],
                         r1 = reinterpret_cast<const float4 *>(rrow + k)[1];
            const int jj[8] = {j0.x, j0.y, j0.z, j0.w, j1.x, j1.y, j1.z, j1.w};
            const float rr[8] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w};
            const int m = min(8, cs - k);
            float thr[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) thr[u] = u < m ? fmaxf(H2i, H2f[jj[u]]) : H2i;
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                if (u < m && exact_in(rr[u], thr[u], jj[u], xi, yi, zi, H2, x, y, z, h, true)) {
                    put(s_b1, k1, orow1, osp1, jj[u]);
                    if (exact_in(rr[u], H2i, jj[u], xi, yi, zi, H2, x, y, z, h, false)) put(s_b0, k0, orow0, osp0, jj[u]);
                }
            }
        }
    }
    for (int q = 0; q < (k0 & 7); ++q) {
        const int k = (k0 & ~7) + q;
        (k < K ? orow0 : osp0)[k] = s_b0[q][t];
    }
    for (int q = 0; q < (k1 & 7); ++q) {
        const int k = (k1 & ~7) + q;
        (k < K ? orow1 : osp1)[k] = s_b1[q][t];
    }
    ocnt0[i] = k0;
    ocnt1[i] = k1;
}

// Mixed-precision density straight from the superset: the gather-set
// decision of k_filter<0>, then CalcDensity's sum (force.h:9-23) in FP32
// partial sums of 32 flushed to FP64, FLAG_GI floor and h update in FP64.
__global__ void __launch_bounds__(128)
k_density_sup32(int n, const int *__restrict__ sup, const float *__restrict__ sup_r2, const float *__restrict__ sup_m,
                const int *__restrict__ scnt, RowMap rm, const double *__restrict__ x,
                const double *__restrict__ y, const double *__restrict__ z, const double *__restrict__ m,
                double *__restrict__ h, const double *__restrict__ hsup, double *__restrict__ dens, float dscale,
                int *err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double hi = h[i];
    const double Hi = __dmul_rn(SUPPORT, hi);
    const double H2 = __dmul_rn(Hi, Hi);
    const float H2i = (float)H2;
    const float invH = 1.0f / (float)Hi;
    const double xi = x[i], yi = y[i], zi = z[i];
    const int c_all = scnt[i];
    float acc_h = 0.0f, acc_l = 0.0f;
    // the index row is read only for the rare entries whose FP32 distance is too close to the
    // threshold to decide (exact_in's band); the stream is r^2 and m_j
    for (int seg = 0; seg < 2; ++seg) {
    int c;
    const int64_t b = row_seg(rm, i, seg, c_all, &c);
    if (c <= 0) break;
    const int *row = sup + b;
    const float *rrow = sup_r2 + b;
    const float *mrow = sup_m + b;
    // software-pipelined: the next chunk's four vector loads are in flight while this chunk is summed
    float4 r0 = reinterpret_cast<const float4 *>(rrow)[0], r1 = reinterpret_cast<const float4 *>(rrow)[1];
    float4 m0 = reinterpret_cast<const float4 *>(mrow)[0], m1 = reinterpret_cast<const float4 *>(mrow)[1];
    for (int k = 0; k < c; k += 8) {
        const float rr[8] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w};
        const float mj[8] = {m0.x, m0.y, m0.z, m0.w, m1.x, m1.y, m1.z, m1.w};
        const int m8 = min(8, c - k);
        if (k + 8 < c) {
            r0 = reinterpret_cast<const float4 *>(rrow + k + 8)[0];
            r1 = reinterpret_cast<const float4 *>(rrow + k + 8)[1];
            m0 = reinterpret_cast<const float4 *>(mrow + k + 8)[0];
            m1 = reinterpret_cast<const float4 *>(mrow + k + 8)[1];
        }
        // every member goes straight into the compensated pair: the sum depends only on the
        // sequence of members (the walk's order), not on where non-members sit in the row, so a
        // row rebuilt with another skin (a repair, another run's violators) gives the same result
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            if (u >= m8) continue;
            bool in = rr[u] < H2i * (1.0f - 1.9073486328125e-06f);
            if (!in && !(rr[u] > H2i * (1.0f + 1.9073486328125e-06f)))
                in = exact_in(rr[u], H2i, row[k + u], xi, yi, zi, H2, x, y, z, h, false);
            if (!in) continue;
            const float s_ = sqrt_a(rr[u]) * invH;
            const float p = fmaxf(1.0f - s_, 0.0f);
            const float p2 = p * p, p4 = p2 * p2;
            df_add(acc_h, acc_l, mj[u] * ((1.0f + s_ * (8.0f + s_ * (25.0f + s_ * 32.0f))) * (p4 * p4)));
        }
    }
    }
    density_tail32(acc_h + acc_l, invH, dscale, m[i], dens + i, h + i);
}

// Every density pass of a step (CalcDensity, force.h:9-23, main.cpp:138-139) for a particle
// in one go: the passes only use the particle's own h, and its row holds its gather set as
// long as h <= KAPPA h_sup.  DT threads share a particle (entries 4 sub .. 4 sub + 3 in steps
// of 4 DT; measured at 1M: DT 1 1.07 ms, 2 0.98, 4 0.97 for the four passes before the loop
// below was made branch-free); a particle whose new h leaves the skin stops after that pass, to
// go on once its row is walked again.  The four entries of a chunk are decided first (the rare
// FP64 edge test behind a call), then summed without branches, two at a time in paired FP32
// arithmetic, non-members as zero terms (0.98 -> 0.69 ms at 1M, bit-identical).  Each term
// m_j W_ij is rounded to a multiple of 2^-40 and summed as an integer, so the sum depends on
// neither the order of the terms nor where non-members sit in the row.  The multiple is taken on
// the particle's run's own mass scale (the terms carry the context's, 2^fixd[run] times the
// run's: a power of two), so a run's sums are the same alone and in any mix of runs.  SPLIT:
// every run's masses on its own scale are at most 15, so each term is at most 16 and takes
// sph_fix40_add (FP32 / integer pipes) instead of __float2ll_rn (FP64 pipe); both give the same
// integers.  Blocks of 64 threads (32 particles): 0.67 -> 0.65 ms at 1M against 128.
constexpr int DT = 2;
template <bool SPLIT>
__global__ void __launch_bounds__(64)
k_density_fused32(int n, int n_pass, const int *__restrict__ sup, const float *__restrict__ sup_r2,
                  const float *__restrict__ sup_m, const int *__restrict__ scnt, RowMap rm,
                  const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ z,
                  const double *__restrict__ m, double *__restrict__ h, const double *__restrict__ hsup,
                  double *__restrict__ dens, float dscale, int *__restrict__ npass, int *n_stopped,
                  const int *__restrict__ prun, const int *__restrict__ fixd) {
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = gt / DT, sub = gt % DT;
    if (i >= n) return;   // whole groups leave together
    int p = npass[i];
    if (p >= n_pass) return;
    // the fixed-point grid 2^(fd - 40) on the context's scale is 2^-40 on the run's
    // (powers of two written as bit patterns: exponent fields moved by fd, |fd| <= 60)
    const int fd = fixd[prun[i]];
    const unsigned b1 = SPH_FIX_B1 + ((unsigned)fd << 23), b2 = SPH_FIX_B2 + ((unsigned)fd << 23);
    const float c1 = __uint_as_float(b1), c2 = __uint_as_float(b2);
    const float to_fix = __uint_as_float((unsigned)(127 + 40 - fd) << 23);                         // 2^(40 - fd)
    const double from_fix = __longlong_as_double((long long)(1023 + fd - 40) << 52);               // 2^(fd - 40)
    const unsigned gm = __activemask();
    double hi = h[i];
    const double hs = hsup[i], xi = x[i], yi = y[i], zi = z[i], mi = m[i];
    const int c_all = scnt[i];
    bool stopped = false;
    for (; p < n_pass && !stopped; ++p) {
        const double Hi = __dmul_rn(SUPPORT, hi);
        const double H2 = __dmul_rn(Hi, Hi);
        const float H2i = (float)H2;
        const float invH = 1.0f / (float)Hi;
        const float lo_b = H2i * (1.0f - 1.9073486328125e-06f), hi_b = H2i * (1.0f + 1.9073486328125e-06f);
        long long acc = 0;
        // SPLIT: 32-bit sums of the raw bit patterns of sph_fix40_add's a and b, their offsets
        // (b1, b2 per term, non-members included: a zero term adds exactly the offsets) taken off
        // when they are flushed, after at most SPH_FIX_TERMS terms
        unsigned rH = 0, rL = 0, nt = 0;   // nt: terms in rH / rL
        const f32x2 ih2 = f2_pack(invH, invH), one2 = f2_pack(1.0f, 1.0f), c1_2 = f2_pack(c1, c1),
                    c2_2 = f2_pack(c2, c2), k32 = f2_pack(32.0f, 32.0f), k25 = f2_pack(25.0f, 25.0f),
                    k8 = f2_pack(8.0f, 8.0f);
        for (int seg = 0; seg < 2; ++seg) {
            int c;
            const int64_t b = row_seg(rm, i, seg, c_all, &c);
            if (c <= 0) break;
            const float *rrow = sup_r2 + b, *mrow = sup_m + b;
            // the next chunk's r^2 loads while this chunk is summed (1M, four passes: 0.69 -> 0.67
            // ms; r^2 and m both ahead: 0.68 ms, more registers)
            float4 rn = 4 * sub < c ? *reinterpret_cast<const float4 *>(rrow + 4 * sub) : make_float4(0.f, 0.f, 0.f, 0.f);
            for (int k = 4 * sub; k < c; k += 4 * DT) {
                if (SPLIT) {
                    if (nt == (unsigned)SPH_FIX_TERMS) {
                        acc += sph_fix40_value(rH - nt * b1, rL - nt * b2);
                        rH = rL = nt = 0;
                    }
                    nt += 4;
                }
                const float4 r4 = rn;
                const float4 m4 = *reinterpret_cast<const float4 *>(mrow + k);
                if (k + 4 * DT < c) rn = *reinterpret_cast<const float4 *>(rrow + k + 4 * DT);
                const float rr[4] = {r4.x, r4.y, r4.z, r4.w};
                // members: inside the band by FP32, at its edge by the FP64 test; padding out
                bool in[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    in[u] = k + u < c && rr[u] < lo_b;
                    if (k + u < c && !in[u] && !(rr[u] > hi_b))
                        in[u] = exact_in_call(rr[u], H2i, sup[b + k + u], xi, yi, zi, H2, x, y, z, h);
                }
                // m_j W(s) for two entries at a time, each lane with the roundings of the scalar
                // m * ((1 + s (8 + s (25 + 32 s))) (q^4 q^4)), q = max(1 - s, 0), s = sqrt(r^2) / H
                float t[4];
#pragma unroll
                for (int pr = 0; pr < 2; ++pr) {
                    const f32x2 s2 = f2_mul(f2_pack(sqrt_a(rr[2 * pr]), sqrt_a(rr[2 * pr + 1])), ih2);
                    float qa, qb;
                    f2_unpack(f2_sub(one2, s2), qa, qb);
                    const f32x2 q = f2_pack(fmaxf(qa, 0.0f), fmaxf(qb, 0.0f));
                    const f32x2 q2 = f2_mul(q, q), q4 = f2_mul(q2, q2);
                    const f32x2 poly = f2_fma(s2, f2_fma(s2, f2_fma(s2, k32, k25), k8), one2);
                    const f32x2 mj = pr == 0 ? f2_pack(m4.x, m4.y) : f2_pack(m4.z, m4.w);
                    f2_unpack(f2_mul(mj, f2_mul(poly, f2_mul(q4, q4))), t[2 * pr], t[2 * pr + 1]);
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) t[u] = in[u] ? t[u] : 0.0f;
                if (SPLIT) {
#pragma unroll
                    for (int pr = 0; pr < 2; ++pr) {
                        const f32x2 tt = f2_pack(t[2 * pr], t[2 * pr + 1]);
                        const f32x2 a = f2_add(tt, c1_2);
                        const f32x2 bb = f2_add(f2_sub(tt, f2_sub(a, c1_2)), c2_2);
                        float a0, a1, b0, b1f;
                        f2_unpack(a, a0, a1);
                        f2_unpack(bb, b0, b1f);
                        rH += __float_as_uint(a0) + __float_as_uint(a1);
                        rL += __float_as_uint(b0) + __float_as_uint(b1f);
                    }
                } else {
#pragma unroll
                    for (int u = 0; u < 4; ++u) acc += __float2ll_rn(t[u] * to_fix);
                }
            }
        }
        if (SPLIT) acc += sph_fix40_value(rH - nt * b1, rL - nt * b2);
#pragma unroll
        for (int o = DT / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(gm, acc, o, DT);
        double rho, hn;
        density_tail32((float)((double)acc * from_fix), invH, dscale, mi, &rho, &hn);
        hi = hn;
        if (sub == 0) {
            dens[i] = rho;
            h[i] = hn;
        }
        // the row can miss members of the next pass's set: the same test as k_viol_mark
        stopped = p + 1 < n_pass && hn > (double)KAPPA * hs;
    }
    if (sub == 0) {
        npass[i] = p;
        if (stopped) atomicAdd(n_stopped, 1);
    }
}

__global__ void k_skin_check(int n, const double *h, const double *hsup, int *err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && h[i] > (double)KAPPA * hsup[i]) atomicOr(err, ERR_SKIN);
}


// (2.5 h)^2 as float, rounded up so FP32 superset tests stay conservative
__global__ void k_h2f(int n, const double *h, float *H2f) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double H = SUPPORT * h[i];
    H2f[i] = __double2float_ru(H * H);
}

// double-float positions (hi / lo floats); .w of xh carries the mass x mscale
__global__ void k_pack_pos(int n, const double *x, const double *y, const double *z, const double *m, double mscale,
                           float4 *xh, float4 *xl) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float ax = (float)x[i], ay = (float)y[i], az = (float)z[i];
    xh[i] = make_float4(ax, ay, az, (float)(m[i] * mscale));
    xl[i] = make_float4((float)(x[i] - (double)ax), (float)(y[i] - (double)ay), (float)(z[i] - (double)az), 0.0f);
}

// spill range lengths: rows longer than K take round8(count - K) entries beyond the row block
__global__ void k_spill_need(int n, const int *cnt, int K, int *need, unsigned long long *total) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    int v = 0;
    if (i < n) v = cnt[i] > K ? ((cnt[i] - K + 7) & ~7) : 0;
    if (i <= n) need[i] = v;
    // the sum in 64 bits: the offsets are 32-bit, so a total past 2^31 must be refused, not wrapped
    unsigned long long w = (unsigned long long)v;
    for (int o = 16; o > 0; o >>= 1) w += __shfl_xor_sync(0xffffffffu, w, o);
    if ((threadIdx.x & 31) == 0 && w) atomicAdd(total, w);
}

}  // namespace sph

using namespace sph;

template <class T>
static int dalloc_n(sph_ctx *ctx, T **p, int64_t n) {
    if (*p) cudaFree(*p);
    *p = nullptr;
    cudaError_t e = cudaMalloc((void **)p, sizeof(T) * (size_t)std::max<int64_t>(n, 1));
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return sph_fail(ctx, SPH_ERR_OOM, "device allocation of %lld bytes failed", (long long)(sizeof(T) * n));
    }
    return SPH_OK;
}

// the double-float positions the walks read: in the mixed path the packs of sph_pack_mixed
// (written after every sort, before any walk, with the same split and the same mass in .w),
// in the FP64 path the walk's own
static const float4 *walk_xh(const sph_ctx *ctx) {
    return ctx->cfg.precision == SPH_PREC_MIXED ? ctx->xh : ctx->sup.pxh;
}
static const float4 *walk_xl(const sph_ctx *ctx) {
    return ctx->cfg.precision == SPH_PREC_MIXED ? ctx->xl : ctx->sup.pxl;
}

// h-dependent float copies; called after every density pass and after the sort
int sph_nbr_refresh_h(sph_ctx *ctx) {
    SphSuper &S = ctx->sup;
    const int n = (int)ctx->n;
    k_h2f<<<sph_div_up(n, 256), 256, 0, ctx->stream>>>(n, FLD(ctx->F, SPH_SMTH, ctx->cap), S.H2f);
    ++ctx->launches;
    SPH_CUDA(ctx, cudaGetLastError());
    return SPH_OK;
}

// after the sort: positions as double-float, units, and the superset marked stale
int sph_nbr_prepare(sph_ctx *ctx) {
    SphSuper &S = ctx->sup;
    const int n = (int)ctx->n;
    const int64_t pitch = ((int64_t)n + 31) / 32 * 32;
    if (S.cap_particles < pitch) {
        SPH_TRY(dalloc_n(ctx, &S.pxh, pitch));
        SPH_TRY(dalloc_n(ctx, &S.pxl, pitch));
        SPH_TRY(dalloc_n(ctx, &S.H2f, pitch));
        SPH_TRY(dalloc_n(ctx, &S.hsup, pitch));
        SPH_TRY(dalloc_n(ctx, &S.cnt, pitch));
        SPH_TRY(dalloc_n(ctx, &S.vR, pitch));
        SPH_TRY(dalloc_n(ctx, &S.npass, pitch));
        S.cap_particles = pitch;
    }
    const int64_t cap = ctx->cap;
    if (ctx->cfg.precision != SPH_PREC_MIXED) {   // the mixed path walks on sph_pack_mixed's packs
        k_pack_pos<<<sph_div_up(n, 256), 256, 0, ctx->stream>>>(n, FLD(ctx->F, SPH_X, cap), FLD(ctx->F, SPH_Y, cap),
                                                                FLD(ctx->F, SPH_Z, cap), FLD(ctx->F, SPH_MASS, cap),
                                                                ctx->mscale, S.pxh, S.pxl);
        ++ctx->launches;
    }
    SPH_TRY(sph_nbr_refresh_h(ctx));
    // units
    Tree &t = ctx->tree;
    const int nc = t.n_cell_host;
    const int grid = 2 * ctx->num_sms;
    k_units<false><<<grid, 256, 0, ctx->stream>>>(t.meta, t.start, t.count, t.first_child, t.n_child, t.tmp_cnt,
                                                  nullptr, nullptr);
    ++ctx->launches;
    SPH_TRY(sph_scan_exclusive(ctx, t.tmp_cnt, t.tmp_off, nullptr, nc, ctx->scan.total));
    int tot = 0;
    SPH_CUDA(ctx, cudaMemcpyAsync(&ctx->host_scalars[0], ctx->scan.total, sizeof(int), cudaMemcpyDeviceToHost,
                                  ctx->stream));
    SPH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    std::memcpy(&tot, &ctx->host_scalars[0], sizeof(int));
    if (S.cap_units < tot) {
        S.cap_units = tot + tot / 4 + 64;
        SPH_TRY(dalloc_n(ctx, &S.units, S.cap_units));
        SPH_TRY(dalloc_n(ctx, &S.umark, S.cap_units));
        SPH_TRY(dalloc_n(ctx, &S.uoff, S.cap_units));
        SPH_TRY(dalloc_n(ctx, &S.uidx, S.cap_units));
    }
    if (S.cap_cells < t.cap) {
        S.cap_cells = t.cap;
        SPH_TRY(dalloc_n(ctx, &S.cvR, S.cap_cells));
    }
    k_units<true><<<grid, 256, 0, ctx->stream>>>(t.meta, t.start, t.count, t.first_child, t.n_child, nullptr,
                                                 t.tmp_off, S.units);
    ++ctx->launches;
    SPH_CUDA(ctx, cudaGetLastError());
    S.n_units = tot;
    S.valid = false;
    S.rebuilds_step = 0;
    ctx->lists[0].valid = ctx->lists[1].valid = false;
    return SPH_OK;
}

// walks the units in uidx (or all units when uidx is null); grows the row capacity if needed
static int walk_units(sph_ctx *ctx, const int *uidx, int n_walk) {
    SphSuper &S = ctx->sup;
    const int n = (int)ctx->n;
    const int64_t pitch = n;   // rows: particle i's entries at i * K .. i * K + K - 1
    const int64_t cap = ctx->cap;
    int *meta = ctx->tree.meta;
    Tree &t = ctx->tree;
    if (S.K == 0) S.K = 192;
    S.K = (S.K + 7) & ~7;   // rows start on 32-byte boundaries
    if (!S.uover || S.n_units > S.cap_uover) {
        SPH_TRY(dalloc_n(ctx, &S.uover, S.cap_units));
        SPH_CUDA(ctx, cudaMemsetAsync(S.uover, 0, sizeof(int) * S.cap_units, ctx->stream));
        S.cap_uover = S.cap_units;
    }
    if (S.rebuilds_step > 0) SPH_TRY(sph_tree_refresh_hmax(ctx));   // cell hmax must follow the current h
    S.rebuilds_step += 1;
    for (int attempt = 0; attempt < 4; ++attempt) {
        if (!S.nbr || S.pitch < pitch || S.K_alloc != S.K || S.spill_alloc != S.spill_cap) {
            if (uidx) {   // a partial walk cannot re-layout the rows: the others would be lost
                uidx = nullptr;
                n_walk = S.n_units;
            }
            if (S.K_alloc != S.K || S.pitch < pitch) S.spill_on = false;   // spill offsets follow K and n
            S.main = (int64_t)S.K * pitch;
            const int64_t tot = S.main + S.spill_cap;
            SPH_TRY(dalloc_n(ctx, &S.nbr, tot));
            SPH_TRY(dalloc_n(ctx, &S.r2, tot));
            SPH_TRY(dalloc_n(ctx, &S.m, tot));
            for (int m = 0; m < 2; ++m) {
                SPH_TRY(dalloc_n(ctx, &ctx->lists[m].nbr, tot));
                SPH_TRY(dalloc_n(ctx, &ctx->lists[m].cnt, pitch));
                ctx->lists[m].K = ctx->lists[m].K_alloc = S.K;
                ctx->lists[m].pitch = S.K;   // row stride of the exact lists
            }
            S.pitch = pitch;
            S.K_alloc = S.K;
            S.spill_alloc = S.spill_cap;
        }
        SPH_CUDA(ctx, cudaMemsetAsync(meta + META_ERR, 0, sizeof(int), ctx->stream));
        SPH_CUDA(ctx, cudaMemsetAsync(meta + META_MAXCNT, 0, sizeof(int), ctx->stream));
        const int blocks = (n_walk + NB_WARPS - 1) / NB_WARPS;
        WalkTree T{t.cinfo, t.blo, t.bhi};
        if (blocks > 0) {
            auto walk = S.spill_on ? k_sup_walk<true> : k_sup_walk<false>;
            walk<<<blocks, NB_WARPS * 32, 0, ctx->stream>>>(
                n_walk, S.units, uidx, FLD(ctx->F, SPH_X, cap), FLD(ctx->F, SPH_Y, cap), FLD(ctx->F, SPH_Z, cap),
                FLD(ctx->F, SPH_SMTH, cap), S.hsup, walk_xh(ctx), walk_xl(ctx), S.H2f, ctx->runs.prun, T, S.nbr, S.r2, S.m,
                S.cnt, S.map(), S.uover, meta + META_ERR, meta + META_MAXCNT);
            ++ctx->launches;
        }
        SPH_CUDA(ctx, cudaGetLastError());
        int *hs = (int *)ctx->host_scalars;
        SPH_CUDA(ctx, cudaMemcpyAsync(hs, meta + META_ERR, 4 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        SPH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        const int errw = hs[0], maxc = hs[META_MAXCNT - META_ERR];
        if (errw & ERR_SPH_STACK) return sph_fail(ctx, SPH_ERR_CAPACITY, "SPH walk stack overflow");
        if (errw & ERR_SPH_LIST_OVERFLOW) {
            if (maxc <= ROW_K_MAX && !S.spill_on) {
                // every row fits a wider block: grow K and rebuild everything
                S.K = std::min(ROW_K_MAX, (maxc + maxc / 4 + 16 + 7) & ~7);
                uidx = nullptr;
                n_walk = S.n_units;
                continue;
            }
            // rows longer than K (the true counts are in cnt) get spill ranges; the units holding
            // them are walked again (all of them if the spill block had to grow)
            if (!S.soff || S.cap_soff < n + 1) {
                SPH_TRY(dalloc_n(ctx, &S.soff, n + 1 + 1024));
                SPH_TRY(dalloc_n(ctx, &S.need, n + 1 + 1024));
                S.cap_soff = n + 1 + 1024;
            }
            unsigned long long *tot64 = reinterpret_cast<unsigned long long *>(ctx->scratch_d);
            SPH_CUDA(ctx, cudaMemsetAsync(tot64, 0, sizeof(unsigned long long), ctx->stream));
            k_spill_need<<<sph_div_up(n + 1, 256), 256, 0, ctx->stream>>>(n, S.cnt, S.K, S.need, tot64);
            ++ctx->launches;
            SPH_CUDA(ctx, cudaMemcpyAsync(&ctx->host_scalars[1], tot64, sizeof(unsigned long long),
                                          cudaMemcpyDeviceToHost, ctx->stream));
            SPH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            unsigned long long need64 = 0;
            std::memcpy(&need64, &ctx->host_scalars[1], sizeof(need64));
            if (need64 > (unsigned long long)INT32_MAX - 4096)
                return sph_fail(ctx, SPH_ERR_CAPACITY,
                                "neighbour rows need %llu entries beyond the row block (smoothing lengths out of "
                                "range?)", need64);
            SPH_TRY(sph_scan_exclusive(ctx, S.need, S.soff, nullptr, n + 1, ctx->scan.total));
            const int64_t need = (int64_t)need64;
            S.spill_on = true;
            S.spilled = need;
            if (need > S.spill_cap) {
                S.spill_cap = need + need / 2 + 4096;   // reallocated at the top of the loop, rows rebuilt
                continue;
            }
            const int grid = 2 * ctx->num_sms;
            SPH_TRY(sph_scan_exclusive(ctx, S.uover, S.uoff, nullptr, S.n_units, ctx->scan.total));
            k_unit_compact<<<grid, 256, 0, ctx->stream>>>(S.n_units, S.uover, S.uoff, S.uidx);
            ++ctx->launches;
            SPH_CUDA(ctx, cudaMemcpyAsync(hs, ctx->scan.total, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
            SPH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            uidx = S.uidx;
            n_walk = hs[0];
            continue;
        }
        S.valid = true;
        if (uidx) S.repairs += 1;
        else S.rebuilds += 1;
        S.units_walked += n_walk;
        return SPH_OK;
    }
    return sph_fail(ctx, SPH_ERR_CAPACITY, "SPH superset capacity could not be grown");
}

// a full walk after a sort: the previous spill layout belongs to the previous order
static int build_superset(sph_ctx *ctx) {
    ctx->sup.spill_on = false;
    return walk_units(ctx, nullptr, ctx->sup.n_units);
}

// makes the superset valid for the current h: full walk after a sort, otherwise a repair of
// the units within reach of particles whose h outgrew the skin
static int ensure_superset(sph_ctx *ctx) {
    SphSuper &S = ctx->sup;
    if (!S.valid) return build_superset(ctx);
    const int n = (int)ctx->n;
    const int64_t cap = ctx->cap;
    int *meta = ctx->tree.meta;
    Tree &t = ctx->tree;
    float *vR = S.vR;
    SPH_CUDA(ctx, cudaMemsetAsync(meta + META_ERR + 8, 0, sizeof(int), ctx->stream));
    k_viol_mark<<<sph_div_up(n, 256), 256, 0, ctx->stream>>>(n, FLD(ctx->F, SPH_SMTH, cap), S.hsup, vR,
                                                              meta + META_ERR + 8);
    ++ctx->launches;
    int *hs = (int *)ctx->host_scalars;
    SPH_CUDA(ctx, cudaMemcpyAsync(hs, meta + META_ERR + 8, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    SPH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const int nviol = hs[0];
    if (nviol == 0) return SPH_OK;
    S.violators += nviol;
    if ((int64_t)nviol * 8 > n) return build_superset(ctx);   // widespread growth: walk everything
    // influence radius per cell, bottom-up
    const int grid = 2 * ctx->num_sms;
    for (int l = t.depth; l >= 0; --l) {
        k_cell_vmax<<<grid, 128, 0, ctx->stream>>>(l, meta, vR, t.cinfo, S.cvR);
        ++ctx->launches;
    }
    const int blocks = (S.n_units + NB_WARPS - 1) / NB_WARPS;
    k_unit_mark<<<blocks, NB_WARPS * 32, 0, ctx->stream>>>(S.n_units, S.units, walk_xh(ctx), walk_xl(ctx), vR, S.cvR,
                                                           t.cinfo, t.blo, t.bhi, ctx->runs.prun, S.umark);
    ++ctx->launches;
    SPH_TRY(sph_scan_exclusive(ctx, S.umark, S.uoff, nullptr, S.n_units, ctx->scan.total));
    k_unit_compact<<<grid, 256, 0, ctx->stream>>>(S.n_units, S.umark, S.uoff, S.uidx);
    ++ctx->launches;
    SPH_CUDA(ctx, cudaMemcpyAsync(hs, ctx->scan.total, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    SPH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const int nmark = hs[0];
    return walk_units(ctx, S.uidx, nmark);
}

// exact list of `mode` (0 gather, 1 symmetric, 2 both) for the current h
int sph_build_sph_lists(sph_ctx *ctx, int mode) {
    SphSuper &S = ctx->sup;
    const int n = (int)ctx->n;
    const int64_t cap = ctx->cap;
    int *meta = ctx->tree.meta;
    SPH_TRY(ensure_superset(ctx));
    if (mode == 2) {   // both lists in one pass
        SphLists &L0 = ctx->lists[0], &L1 = ctx->lists[1];
        k_filter2<<<sph_div_up(n, 128), 128, 0, ctx->stream>>>(
            n, S.nbr, S.r2, S.cnt, S.map(), FLD(ctx->F, SPH_X, cap), FLD(ctx->F, SPH_Y, cap), FLD(ctx->F, SPH_Z, cap),
            FLD(ctx->F, SPH_SMTH, cap), S.H2f, L0.nbr, L0.cnt, L1.nbr, L1.cnt);
        ++ctx->launches;
        SPH_CUDA(ctx, cudaGetLastError());
        L0.valid = L1.valid = true;
        return SPH_OK;
    }
    SphLists &L = ctx->lists[mode];
    if (mode == 0)
        k_filter<0><<<sph_div_up(n, 128), 128, 0, ctx->stream>>>(
            n, S.nbr, S.r2, S.cnt, S.map(), FLD(ctx->F, SPH_X, cap), FLD(ctx->F, SPH_Y, cap), FLD(ctx->F, SPH_Z, cap),
            FLD(ctx->F, SPH_SMTH, cap), S.hsup, S.H2f, L.nbr, L.cnt, meta + META_ERR);
    else
        k_filter<1><<<sph_div_up(n, 128), 128, 0, ctx->stream>>>(
            n, S.nbr, S.r2, S.cnt, S.map(), FLD(ctx->F, SPH_X, cap), FLD(ctx->F, SPH_Y, cap), FLD(ctx->F, SPH_Z, cap),
            FLD(ctx->F, SPH_SMTH, cap), S.hsup, S.H2f, L.nbr, L.cnt, meta + META_ERR);
    ++ctx->launches;
    SPH_CUDA(ctx, cudaGetLastError());
    L.valid = true;
    return SPH_OK;
}

// mixed-precision density pass straight from the superset (no exact list)
int sph_density_from_superset(sph_ctx *ctx) {
    SphSuper &S = ctx->sup;
    const int n = (int)ctx->n;
    const int64_t cap = ctx->cap;
    int *meta = ctx->tree.meta;
    SPH_TRY(ensure_superset(ctx));
    k_density_sup32<<<sph_div_up(n, 128), 128, 0, ctx->stream>>>(
        n, S.nbr, S.r2, S.m, S.cnt, S.map(), FLD(ctx->F, SPH_X, cap), FLD(ctx->F, SPH_Y, cap),
        FLD(ctx->F, SPH_Z, cap), FLD(ctx->F, SPH_MASS, cap), FLD(ctx->F, SPH_SMTH, cap), S.hsup,
        FLD(ctx->F, SPH_DENS, cap), (float)(1365.0 / 64.0 / (3.141592653589793 * ctx->mscale)), meta + META_ERR);
    ++ctx->launches;
    SPH_CUDA(ctx, cudaGetLastError());
    ctx->lists[0].valid = false;
    return sph_nbr_refresh_h(ctx);
}

int sph_nbr_ensure_superset(sph_ctx *ctx) { return ensure_superset(ctx); }

// all density passes of the mixed path: rounds of k_density_fused32, the rows of the particles
// that left their skin walked again between rounds (each round takes every unfinished particle
// at least one pass further, so there are at most n_dens_iter rounds)
int sph_density_fused(sph_ctx *ctx) {
    SphSuper &S = ctx->sup;
    const int n = (int)ctx->n;
    const int64_t cap = ctx->cap;
    const int np = ctx->cfg.n_dens_iter;
    int *stopped = ctx->tree.meta + META_ERR + 9;
    int *hs = (int *)ctx->host_scalars;
    SPH_CUDA(ctx, cudaMemsetAsync(S.npass, 0, sizeof(int) * n, ctx->stream));
    for (int round = 0; round <= np; ++round) {
        SPH_TRY(ensure_superset(ctx));
        SPH_TRY(time_mark(ctx, SEG_DENS_LIST));
        SPH_CUDA(ctx, cudaMemsetAsync(stopped, 0, sizeof(int), ctx->stream));
        auto kd = ctx->runs.fix_split ? k_density_fused32<true> : k_density_fused32<false>;
        kd<<<sph_div_up((int64_t)n * DT, 64), 64, 0, ctx->stream>>>(
            n, np, S.nbr, S.r2, S.m, S.cnt, S.map(), FLD(ctx->F, SPH_X, cap), FLD(ctx->F, SPH_Y, cap),
            FLD(ctx->F, SPH_Z, cap), FLD(ctx->F, SPH_MASS, cap), FLD(ctx->F, SPH_SMTH, cap), S.hsup,
            FLD(ctx->F, SPH_DENS, cap), (float)(1365.0 / 64.0 / (3.141592653589793 * ctx->mscale)), S.npass,
            stopped, ctx->runs.prun, ctx->runs.fixd);
        ++ctx->launches;
        SPH_CUDA(ctx, cudaGetLastError());
        SPH_TRY(time_mark(ctx, SEG_DENS));
        SPH_CUDA(ctx, cudaMemcpyAsync(hs, stopped, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        SPH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        SPH_TRY(sph_nbr_refresh_h(ctx));   // H2f of the current h, for the walks and the filters
        if (hs[0] == 0) break;
        if (round == np) return sph_fail(ctx, SPH_ERR_STATE, "density passes did not converge over the skin repairs");
    }
    ctx->lists[0].valid = false;
    return SPH_OK;
}
