// Pair-interaction passes, EoS, integrator and reductions.
//
// FP64 path: one thread per i-particle over its exact neighbour list (ELL),
// arithmetic as in the reference functors (force.h:9-23, 89-106, 113-147,
// 154-168); j is summed in ascending key order, the order the oracle uses.
//
// Mixed path (SPH_PREC_MIXED): the same lists and epilogues, with the pair
// arithmetic in FP32 on double-float positions / velocities (hi + lo floats,
// so x_i - x_j is formed without FP64 arithmetic), partial sums of at most
// 32 neighbours (SPH) or one shared-memory tile of j (gravity) accumulated in
// FP32 and flushed into double-float or FP64 accumulators.  Epilogues
// (density floor, h update, grad-h normalisation, Balsara, dt), the EoS, the
// integrator and every reduction stay in FP64.
#include "sph_physics.cuh"

namespace sph {

constexpr int PT = 128;   // threads per block for per-particle kernels

// ---------------------------------------------------------------------------
// FP64 density, CalcDensity (force.h:9-23) + FLAG_GI floor + h update

__global__ void __launch_bounds__(PT) k_density64(int n, const double *__restrict__ x, const double *__restrict__ y,
                                                  const double *__restrict__ z, const double *__restrict__ m,
                                                  double *__restrict__ h, double *__restrict__ dens,
                                                  const int *__restrict__ nbr, const int *__restrict__ cnt,
                                                  RowMap rm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double xi = x[i], yi = y[i], zi = z[i], hi = h[i];
    const double H = SUPPORT * hi;
    const double invH = 1.0 / H;
    const double norm = kernel_norm(H);
    double sum = 0.0;
    for (int seg = 0, c; seg < 2; ++seg) {
    const int *row = nbr + row_seg(rm, i, seg, cnt[i], &c);
    for (int k = 0; k < c; ++k) {
        const int j = row[k];
        const double dx = x[j] - xi, dy = y[j] - yi, dz = z[j] - zi;
        const double r = sqrt(dx * dx + dy * dy + dz * dz);
        double w, g;
        wendland_poly(r * invH, w, g);
        sum += m[j] * w;
    }
    }
    const double d = fmax(DENS_FLOOR, sum * norm);
    dens[i] = d;
    h[i] = SMTH_COEF * pow(m[i] / d, 1.0 / 3.0);
}

// ---------------------------------------------------------------------------
// EoS, CalcPressure (force.h:26-32)

__global__ void k_eos(int n, const DevMaterial *__restrict__ mats, const int32_t *__restrict__ mat,
                      const double *__restrict__ dens, const double *__restrict__ eng, double *__restrict__ pres,
                      double *__restrict__ snds) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double P, cs;
    eos_eval(mats[mat[i]], dens[i], eng[i], P, cs);
    pres[i] = P;
    snds[i] = cs;
}

// ---------------------------------------------------------------------------
// FP64 derivative, CalcDerivative (force.h:89-106) + Balsara (class.h:132-142)

struct DrvtArgs {
    const double *x, *y, *z, *vx, *vy, *vz, *m, *h, *dens, *snds;
    double *divv, *rx, *ry, *rz, *gradh, *bal;
    const int *nbr, *cnt;
    RowMap rm;
};

__global__ void __launch_bounds__(PT) k_drvt64(int n, DrvtArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double xi = a.x[i], yi = a.y[i], zi = a.z[i], ux = a.vx[i], uy = a.vy[i], uz = a.vz[i];
    const double hi = a.h[i], rhoi = a.dens[i];
    const double H = SUPPORT * hi, invH = 1.0 / H, norm = kernel_norm(H), ceps = 1.0e-6 * hi;
    double dv = 0.0, r0 = 0.0, r1 = 0.0, r2 = 0.0, gs = 0.0;
    for (int seg = 0, c; seg < 2; ++seg) {
    const int *row = a.nbr + row_seg(a.rm, i, seg, a.cnt[i], &c);
    for (int k = 0; k < c; ++k) {
        const int j = row[k];
        const double dx = xi - a.x[j], dy = yi - a.y[j], dz = zi - a.z[j];
        const double mj = a.m[j];
        const double ax = -mj * (ux - a.vx[j]), ay = -mj * (uy - a.vy[j]), az = -mj * (uz - a.vz[j]);
        const double rr2 = dx * dx + dy * dy + dz * dz;
        const double r = sqrt(rr2);
        double w, g;
        wendland_poly(r * invH, w, g);
        const double gf = norm * g / (r * H + ceps);     // gradW = dr * gf (kernel.h:22-34)
        dv += gf * (ax * dx + ay * dy + az * dz);
        r0 += gf * (ay * dz - az * dy);
        r1 += gf * (az * dx - ax * dz);
        r2 += gf * (ax * dy - ay * dx);
        gs += mj * (3.0 * norm * w + gf * rr2);
    }
    }
    gs = -gs / hi;
    gs = 1.0 / (1.0 + hi * gs / (3.0 * rhoi));
    dv /= rhoi;
    r0 /= rhoi;
    r1 /= rhoi;
    r2 /= rhoi;
    a.divv[i] = dv;
    a.rx[i] = r0;
    a.ry[i] = r1;
    a.rz[i] = r2;
    a.gradh[i] = gs;
    a.bal[i] = fabs(dv) / (fabs(dv) + sqrt(r0 * r0 + r1 * r1 + r2 * r2) + 1.0e-4 * a.snds[i] / hi);
}

// ---------------------------------------------------------------------------
// FP64 hydro, CalcHydroForce (force.h:113-147)

struct HydroArgs {
    const double *x, *y, *z, *vx, *vy, *vz, *m, *h, *dens, *pres, *snds, *gradh, *bal;
    const double4 *aux;   // per particle: invH, norm, 1e-6 h, f P / rho^2
    double *ax, *ay, *az, *edot, *dt;
    const int *nbr, *cnt;
    RowMap rm;
};

__global__ void k_hydro_aux64(int n, const double *h, const double *dens, const double *pres, const double *gradh,
                              double4 *aux) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double hi = h[i], H = SUPPORT * hi;
    aux[i] = make_double4(1.0 / H, kernel_norm(H), 1.0e-6 * hi, gradh[i] * pres[i] / (dens[i] * dens[i]));
}

__global__ void __launch_bounds__(PT) k_hydro64(int n, HydroArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double xi = a.x[i], yi = a.y[i], zi = a.z[i], ux = a.vx[i], uy = a.vy[i], uz = a.vz[i];
    const double hi = a.h[i], rhoi = a.dens[i], ci = a.snds[i], fi = a.gradh[i], bi = a.bal[i];
    const double4 ai = a.aux[i];
    const double Hi = SUPPORT * hi;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, e = 0.0, vmax = 0.0;
    for (int seg = 0, c; seg < 2; ++seg) {
    const int *row = a.nbr + row_seg(a.rm, i, seg, a.cnt[i], &c);
    for (int k = 0; k < c; ++k) {
        const int j = row[k];
        const double dx = xi - a.x[j], dy = yi - a.y[j], dz = zi - a.z[j];
        const double wx = ux - a.vx[j], wy = uy - a.vy[j], wz = uz - a.vz[j];
        const double rr2 = dx * dx + dy * dy + dz * dz;
        const double r = sqrt(rr2);
        const double dvdr = wx * dx + wy * dy + wz * dz;
        const double w = (dvdr < 0) ? dvdr / r : 0.0;
        const double vsig = ci + a.snds[j] - 3.0 * w;
        vmax = fmax(vmax, vsig);
        const double4 aj = a.aux[j];
        const double AV = -AV_STRENGTH * 0.5 * vsig * w / (0.5 * (rhoi + a.dens[j])) * 0.5 * (bi + a.bal[j]);
        double wi_, gi_, wj_, gj_;
        wendland_poly(r * ai.x, wi_, gi_);
        wendland_poly(r * aj.x, wj_, gj_);
        const double Hj = SUPPORT * a.h[j];
        const double gfi = ai.y * gi_ / (r * Hi + ai.z);
        const double gfj = aj.y * gj_ / (r * Hj + aj.z);
        const double gws = 0.5 * (gfi * fi + gfj * a.gradh[j]);
        const double mj = a.m[j];
        const double coef = mj * (ai.w * gfi + aj.w * gfj + AV * gws);
        a0 -= coef * dx;
        a1 -= coef * dy;
        a2 -= coef * dz;
        e += mj * (ai.w + 0.5 * AV) * gws * dvdr;
    }
    }
    a.ax[i] = a0;
    a.ay[i] = a1;
    a.az[i] = a2;
    a.edot[i] = e;
    a.dt[i] = C_CFL * 2.0 * hi / vmax;
}

// ---------------------------------------------------------------------------
// FP64 gravity, CalcGravityForce<EPJ> then <SPJMonopole> (force.h:154-168)

constexpr int GT = 128;

__global__ void __launch_bounds__(GT) k_grav64(const int *__restrict__ group_cell, const int *__restrict__ cstart,
                                               const int *__restrict__ ccount, const double *__restrict__ x,
                                               const double *__restrict__ y, const double *__restrict__ z,
                                               const double *__restrict__ m, const double *__restrict__ h,
                                               const double4 *__restrict__ com, const int *__restrict__ n_epj,
                                               const int *__restrict__ off_epj, const int *__restrict__ epj,
                                               const int *__restrict__ n_spj, const int *__restrict__ off_spj,
                                               const int *__restrict__ spj, double G, double *gx, double *gy,
                                               double *gz, double *pot) {
    __shared__ double4 tile[GT];   // (x, y, z, G m)
    const int g = blockIdx.x;
    const int gc = group_cell[g];
    const int s = cstart[gc], cnt = ccount[gc];
    const int ne = n_epj[g], ns = n_spj[g];
    const int *E = epj + off_epj[g];
    const int *S = spj + off_spj[g];
    for (int i0 = 0; i0 < cnt; i0 += GT) {
        const int i = s + i0 + threadIdx.x;
        const bool act = i0 + threadIdx.x < cnt;
        const double xi = act ? x[i] : 0.0, yi = act ? y[i] : 0.0, zi = act ? z[i] : 0.0;
        const double eps2 = act ? h[i] * h[i] : 1.0;
        double a0 = 0.0, a1 = 0.0, a2 = 0.0, p = 0.0;
        // EPJ then SPJ, each in list order (the two functor calls of main.cpp:145-146)
        for (int pass = 0; pass < 2; ++pass) {
            const int nl = pass == 0 ? ne : ns;
            for (int t0 = 0; t0 < nl; t0 += GT) {
                const int k = t0 + threadIdx.x;
                if (k < nl) {
                    if (pass == 0) {
                        const int j = E[k];
                        tile[threadIdx.x] = make_double4(x[j], y[j], z[j], G * m[j]);
                    } else {
                        const double4 q = com[S[k]];
                        tile[threadIdx.x] = make_double4(q.x, q.y, q.z, G * q.w);
                    }
                }
                __syncthreads();
                const int tn = min(GT, nl - t0);
                for (int t = 0; t < tn; ++t) {
                    const double4 q = tile[t];
                    const double dx = xi - q.x, dy = yi - q.y, dz = zi - q.z;
                    const double dri = rsqrt(fma(dx, dx, fma(dy, dy, fma(dz, dz, eps2))));
                    const double gmr = q.w * dri;
                    const double gmr3 = gmr * (dri * dri);
                    a0 = fma(-gmr3, dx, a0);
                    a1 = fma(-gmr3, dy, a1);
                    a2 = fma(-gmr3, dz, a2);
                    p -= gmr;
                }
                __syncthreads();
            }
        }
        if (act) {
            gx[i] = a0;
            gy[i] = a1;
            gz[i] = a2;
            pot[i] = p;
        }
    }
}

// ---------------------------------------------------------------------------
// Mixed precision: double-float packing

// split_df: sph_physics.cuh

// positions + scaled mass, velocities + h; called after the sort (and h refresh)
__global__ void k_pack_df(int n, const double *x, const double *y, const double *z, const double *vx,
                          const double *vy, const double *vz, const double *m, const double *h, double mscale,
                          float4 *xh, float4 *xl, float4 *vh, float4 *vl) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float a, b, c, d, e, f;
    split_df(x[i], a, d);
    split_df(y[i], b, e);
    split_df(z[i], c, f);
    xh[i] = make_float4(a, b, c, (float)(m[i] * mscale));
    xl[i] = make_float4(d, e, f, (float)h[i]);
    split_df(vx[i], a, d);
    split_df(vy[i], b, e);
    split_df(vz[i], c, f);
    vh[i] = make_float4(a, b, c, 0.0f);
    vl[i] = make_float4(d, e, f, 0.0f);
}

__device__ __forceinline__ float df_diff(float ah, float al, float bh, float bl) { return (ah - bh) + (al - bl); }

// mixed density
__global__ void __launch_bounds__(PT) k_density32(int n, const float4 *__restrict__ xh, const float4 *__restrict__ xl,
                                                  const double *__restrict__ m, double *__restrict__ h,
                                                  double *__restrict__ dens, const int *__restrict__ nbr,
                                                  const int *__restrict__ cnt, RowMap rm, float dscale) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 pih = xh[i], pil = xl[i];
    const double hi = h[i];
    const double H = SUPPORT * hi;
    const float invH = 1.0f / (float)H;
    float acc_h = 0.0f, acc_l = 0.0f;
    float part = 0.0f;
    const RowView row = row_view(nbr, rm, i, cnt[i]);
    for (int k = 0; k < row.c; ++k) {
        const int j = *row.at(k);
        const float4 qh = xh[j], ql = xl[j];
        const float dx = df_diff(qh.x, ql.x, pih.x, pil.x);
        const float dy = df_diff(qh.y, ql.y, pih.y, pil.y);
        const float dz = df_diff(qh.z, ql.z, pih.z, pil.z);
        const float r = sqrt_a(dx * dx + dy * dy + dz * dz);
        float w, g;
        wendland_poly_f(r * invH, w, g);
        part = fmaf(qh.w, w, part);
        if ((k & 31) == 31) {
            df_add(acc_h, acc_l, part);
            part = 0.0f;
        }
    }
    df_add(acc_h, acc_l, part);
    density_tail32(acc_h + acc_l, invH, dscale, m[i], dens + i, h + i);
}

// mixed derivative
struct DrvtArgs32 {
    const float4 *xh, *xl, *vh, *vl;
    const double *h, *dens, *snds;
    double *divv, *rx, *ry, *rz, *gradh, *bal;
    const int *nbr, *cnt;
    RowMap rm;
    float kscale;   // (1365/64) / (pi mscale)
};

__device__ __forceinline__ void drvt_pair32(const float4 pih, const float4 pil, const float4 vih, const float4 vil,
                                            const float4 qh, const float4 ql, const float4 uh, const float4 ul,
                                            float invH, float Hf, float ceps, float P[5]) {
    const float dx = df_diff(pih.x, pil.x, qh.x, ql.x);
    const float dy = df_diff(pih.y, pil.y, qh.y, ql.y);
    const float dz = df_diff(pih.z, pil.z, qh.z, ql.z);
    const float wx = df_diff(vih.x, vil.x, uh.x, ul.x);
    const float wy = df_diff(vih.y, vil.y, uh.y, ul.y);
    const float wz = df_diff(vih.z, vil.z, uh.z, ul.z);
    const float rr2 = dx * dx + dy * dy + dz * dz;
    const float r = sqrt_a(rr2);
    float w, g;
    wendland_poly_f(r * invH, w, g);
    const float gf = g * rcp_a(r * Hf + ceps);
    const float mg = -qh.w * gf;
    P[0] = fmaf(mg, wx * dx + wy * dy + wz * dz, P[0]);
    P[1] = fmaf(mg, wy * dz - wz * dy, P[1]);
    P[2] = fmaf(mg, wz * dx - wx * dz, P[2]);
    P[3] = fmaf(mg, wx * dy - wy * dx, P[3]);
    P[4] = fmaf(qh.w, 3.0f * w + gf * rr2, P[4]);
}

// TPI threads share one i-particle: thread `sub` takes the neighbour pairs 2 sub, 2 sub + 2 TPI, ...
// and the compensated partial sums are combined by shuffles (TPI = 1: one thread per particle)
template <int TPI>
__device__ __forceinline__ void df_group_sum(float &hi, float &lo) {
    const unsigned m = __activemask();
#pragma unroll
    for (int off = TPI / 2; off > 0; off >>= 1) {
        const float oh = __shfl_xor_sync(m, hi, off, TPI), ol = __shfl_xor_sync(m, lo, off, TPI);
        df_add(hi, lo, oh);
        lo += ol;
    }
}

template <int TPI>
__global__ void __launch_bounds__(PT) k_drvt32(int n, DrvtArgs32 a) {
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = gt / TPI, sub = gt % TPI;
    if (i >= n) return;   // whole groups of TPI lanes leave together
    const float4 pih = a.xh[i], pil = a.xl[i], vih = a.vh[i], vil = a.vl[i];
    const double hi = a.h[i];
    const float Hf = (float)(SUPPORT * hi), invH = 1.0f / Hf, ceps = (float)(1.0e-6 * hi);
    // kernel normalisation folded out of the pair sums and applied once at the end
    float Dh[5] = {0, 0, 0, 0, 0}, Dl[5] = {0, 0, 0, 0, 0};
    float P[5] = {0, 0, 0, 0, 0};
    const RowView row = row_view(a.nbr, a.rm, i, a.cnt[i]);
    const int c = row.c;
    int k = 2 * sub, it = 0;
    for (; k + 2 <= c; k += 2 * TPI) {
        const int2 jp = *reinterpret_cast<const int2 *>(row.at(k));
        const int j0 = jp.x, j1 = jp.y;
        const float4 qh0 = a.xh[j0], ql0 = a.xl[j0], uh0 = a.vh[j0], ul0 = a.vl[j0];
        const float4 qh1 = a.xh[j1], ql1 = a.xl[j1], uh1 = a.vh[j1], ul1 = a.vl[j1];
        drvt_pair32(pih, pil, vih, vil, qh0, ql0, uh0, ul0, invH, Hf, ceps, P);
        drvt_pair32(pih, pil, vih, vil, qh1, ql1, uh1, ul1, invH, Hf, ceps, P);
        if ((++it & 15) == 0) {
#pragma unroll
            for (int q = 0; q < 5; ++q) {
                df_add(Dh[q], Dl[q], P[q]);
                P[q] = 0.0f;
            }
        }
    }
    if (k < c) {
        const int j = *row.at(k);
        drvt_pair32(pih, pil, vih, vil, a.xh[j], a.xl[j], a.vh[j], a.vl[j], invH, Hf, ceps, P);
    }
    // per-particle tail of force.h:70-76 in FP32
    const float sc = a.kscale * (invH * invH * invH);
    float D[5];
#pragma unroll
    for (int q = 0; q < 5; ++q) {
        df_add(Dh[q], Dl[q], P[q]);
        if (TPI > 1) df_group_sum<TPI>(Dh[q], Dl[q]);
        D[q] = (Dh[q] + Dl[q]) * sc;
    }
    if (sub != 0) return;
    const float rho = (float)a.dens[i], hf = (float)hi;
    const float gs = 1.0f / (1.0f + hf * (-D[4] / hf) / (3.0f * rho));
    const float dv = D[0] / rho, r0 = D[1] / rho, r1 = D[2] / rho, r2 = D[3] / rho;
    a.divv[i] = dv;
    a.rx[i] = r0;
    a.ry[i] = r1;
    a.rz[i] = r2;
    a.gradh[i] = gs;
    a.bal[i] = fabsf(dv) / (fabsf(dv) + sqrtf(r0 * r0 + r1 * r1 + r2 * r2) + 1.0e-4f * (float)a.snds[i] / hf);
}

// mixed hydro: per-particle FP32 pack hA = (f P / rho^2, c_s, f, Bal), and rho, 1/H and h in the
// free .w slots of the velocity and position packs (vh.w, vl.w, xl.w), so a neighbour's data is
// five float4 (80 B) gathered; H and 1e-6 h follow from h (hydro_b).  The i-particle's kernel
// normalisation is factored out of the FP32 sums and applied in FP64; the j-particle's enters
// as the ratio (H_i / H_j)^3.
__global__ void k_hydro_pack32(int n, const double *h, const double *dens, const double *pres, const double *snds,
                               const double *gradh, const double *bal, float4 *hA, float4 *xl, float4 *vh,
                               float4 *vl) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float hi = (float)h[i], H = __fmul_rn((float)SUPPORT, hi), rho = (float)dens[i], f = (float)gradh[i];
    hA[i] = make_float4(f * (float)pres[i] / (rho * rho), (float)snds[i], f, (float)bal[i]);
    reinterpret_cast<float *>(xl + i)[3] = hi;
    reinterpret_cast<float *>(vh + i)[3] = rho;
    reinterpret_cast<float *>(vl + i)[3] = 1.0f / H;
}

// (rho, 1/H, H, 1e-6 h) of a particle from its packs (the products not fused into later sums)
__device__ __forceinline__ float4 hydro_b(const float4 &xl, const float4 &vh, const float4 &vl) {
    return make_float4(vh.w, vl.w, __fmul_rn((float)SUPPORT, xl.w), __fmul_rn(1.0e-6f, xl.w));
}

struct HydroArgs32 {
    const float4 *xh, *xl, *vh, *vl, *hA;
    const double *h;
    double *ax, *ay, *az, *edot, *dt;
    const int *nbr, *cnt;
    RowMap rm;
    float kscale;   // (1365/64) / (pi mscale)
};

struct HydroJ32 {
    float4 qh, ql, uh, ul, A, B;
};

__device__ __forceinline__ void hydro_pair32(const float4 pih, const float4 pil, const float4 vih, const float4 vil,
                                             const float4 Ai, const float4 Bi, const HydroJ32 &J, float P[4],
                                             float &vmax) {
    const float dx = df_diff(pih.x, pil.x, J.qh.x, J.ql.x);
    const float dy = df_diff(pih.y, pil.y, J.qh.y, J.ql.y);
    const float dz = df_diff(pih.z, pil.z, J.qh.z, J.ql.z);
    const float wx = df_diff(vih.x, vil.x, J.uh.x, J.ul.x);
    const float wy = df_diff(vih.y, vil.y, J.uh.y, J.ul.y);
    const float wz = df_diff(vih.z, vil.z, J.uh.z, J.ul.z);
    const float rr2 = dx * dx + dy * dy + dz * dz;
    const float r = sqrt_a(rr2);   // 0 for the particle itself
    const float dvdr = wx * dx + wy * dy + wz * dz;
    const float w = (dvdr < 0.0f) ? dvdr * rcp_a(r) : 0.0f;   // dvdr < 0 implies r > 0
    const float vsig = Ai.y + J.A.y - 3.0f * w;
    vmax = fmaxf(vmax, vsig);
    const float AV = -0.5f * vsig * w * rcp_a(0.5f * (Bi.x + J.B.x)) * 0.5f * (Ai.w + J.A.w);
    float wi_, gi_, wj_, gj_;
    wendland_poly_f(r * Bi.y, wi_, gi_);
    wendland_poly_f(r * J.B.y, wj_, gj_);
    const float nr = Bi.z * J.B.y;
    const float gfi = gi_ * rcp_a(r * Bi.z + Bi.w);
    const float gfj = (nr * nr * nr) * gj_ * rcp_a(r * J.B.z + J.B.w);
    const float gws = 0.5f * (gfi * Ai.z + gfj * J.A.z);
    const float coef = J.qh.w * (Ai.x * gfi + J.A.x * gfj + AV * gws);
    P[0] = fmaf(-coef, dx, P[0]);
    P[1] = fmaf(-coef, dy, P[1]);
    P[2] = fmaf(-coef, dz, P[2]);
    P[3] = fmaf(J.qh.w * (Ai.x + 0.5f * AV) * gws, dvdr, P[3]);
}

__device__ __forceinline__ HydroJ32 load_hydro_j(const HydroArgs32 &a, int j) {
    HydroJ32 J;
    J.qh = a.xh[j];
    J.ql = a.xl[j];
    J.uh = a.vh[j];
    J.ul = a.vl[j];
    J.A = a.hA[j];
    J.B = hydro_b(J.ql, J.uh, J.ul);
    return J;
}

// six blocks per SM, 80 registers (measured at 1M: 0.91 ms against 0.97 at the 86 registers of
// five blocks, when first tuned; with the index prefetch, 0.74 ms against 0.80 at seven blocks,
// 72 registers and spills)
template <int TPI>
__global__ void __launch_bounds__(PT, 6) k_hydro32(int n, HydroArgs32 a) {
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = gt / TPI, sub = gt % TPI;
    if (i >= n) return;   // whole groups of TPI lanes leave together
    const float4 pih = a.xh[i], pil = a.xl[i], vih = a.vh[i], vil = a.vl[i];
    const float4 Ai = a.hA[i], Bi = hydro_b(pil, vih, vil);
    float Dh[4] = {0, 0, 0, 0}, Dl[4] = {0, 0, 0, 0};
    float P[4] = {0, 0, 0, 0};
    float vmax = 0.0f;
    const RowView row = row_view(a.nbr, a.rm, i, a.cnt[i]);
    const int c = row.c;
    int k = 2 * sub, it = 0;
    // the next pair's indices load while this pair is gathered and summed (1M: 0.79 -> 0.74 ms; the
    // derivative kernel, which gathers 64 B per neighbour instead of 80, gained nothing from it)
    int2 jn = k + 2 <= c ? *reinterpret_cast<const int2 *>(row.at(k)) : make_int2(0, 0);
    for (; k + 2 <= c; k += 2 * TPI) {
        const int2 jp = jn;
        if (k + 2 * TPI + 2 <= c) jn = *reinterpret_cast<const int2 *>(row.at(k + 2 * TPI));
        const int j0 = jp.x, j1 = jp.y;
        const HydroJ32 J0 = load_hydro_j(a, j0), J1 = load_hydro_j(a, j1);
        hydro_pair32(pih, pil, vih, vil, Ai, Bi, J0, P, vmax);
        hydro_pair32(pih, pil, vih, vil, Ai, Bi, J1, P, vmax);
        if ((++it & 15) == 0) {
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                df_add(Dh[q], Dl[q], P[q]);
                P[q] = 0.0f;
            }
        }
    }
    if (k < c) {
        const HydroJ32 J = load_hydro_j(a, *row.at(k));
        hydro_pair32(pih, pil, vih, vil, Ai, Bi, J, P, vmax);
    }
    // kernel normalisation of i (Bi.y = 1 / H_i) and the mass scale, in FP32
    const float sc = a.kscale * (Bi.y * Bi.y * Bi.y);
    float D[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        df_add(Dh[q], Dl[q], P[q]);
        if (TPI > 1) df_group_sum<TPI>(Dh[q], Dl[q]);
        D[q] = (Dh[q] + Dl[q]) * sc;
    }
    if (TPI > 1) {
        const unsigned m = __activemask();
        for (int off = TPI / 2; off > 0; off >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(m, vmax, off, TPI));
    }
    if (sub != 0) return;
    a.ax[i] = D[0];
    a.ay[i] = D[1];
    a.az[i] = D[2];
    a.edot[i] = D[3];
    a.dt[i] = (float)(2.0 * C_CFL) * (float)a.h[i] / vmax;   // force.h:126
}

// cell monopoles as double-float with G folded into the mass
__global__ void k_pack_cells32(const int *meta, const double4 *com, double G, double gscale, float4 *ch, float4 *cl) {
    const int nc = meta[MAX_LEVELS];
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        const double4 q = com[c];
        float a, b, cc, d, e, f;
        split_df(q.x, a, d);
        split_df(q.y, b, e);
        split_df(q.z, cc, f);
        ch[c] = make_float4(a, b, cc, (float)(G * q.w * gscale));
        cl[c] = make_float4(d, e, f, 0.0f);
    }
}

__global__ void __launch_bounds__(GT) k_grav32(const int *__restrict__ group_cell, const int *__restrict__ cstart,
                                               const int *__restrict__ ccount, const float4 *__restrict__ xh,
                                               const float4 *__restrict__ xl, const double *__restrict__ m,
                                               const double *__restrict__ h, const float4 *__restrict__ ch,
                                               const float4 *__restrict__ cl, const int *__restrict__ n_epj,
                                               const int *__restrict__ off_epj, const int *__restrict__ epj,
                                               const int *__restrict__ n_spj, const int *__restrict__ off_spj,
                                               const int *__restrict__ spj, double G, double gscale,
                                               double inv_gscale, double *gx, double *gy, double *gz,
                                               double *pot) {
    __shared__ float4 tile[GT];
    const int g = blockIdx.x;
    const int gc = group_cell[g];
    const int s = cstart[gc], cnt = ccount[gc];
    const int ne = n_epj[g], ns = n_spj[g];
    const int *E = epj + off_epj[g];
    const int *S = spj + off_spj[g];
    const float4 c_h = xh[s], c_l = xl[s];     // group origin (its first particle)
    for (int i0 = 0; i0 < cnt; i0 += GT) {
        const int i = s + i0 + threadIdx.x;
        const bool act = i0 + threadIdx.x < cnt;
        float xi = 0.f, yi = 0.f, zi = 0.f, eps2 = 1.f;
        if (act) {
            const float4 ph = xh[i], pl = xl[i];
            xi = df_diff(ph.x, pl.x, c_h.x, c_l.x);
            yi = df_diff(ph.y, pl.y, c_h.y, c_l.y);
            zi = df_diff(ph.z, pl.z, c_h.z, c_l.z);
            const double hh = h[i];
            eps2 = (float)(hh * hh);
        }
        double D[4] = {0, 0, 0, 0};
        for (int pass = 0; pass < 2; ++pass) {
            const int nl = pass == 0 ? ne : ns;
            for (int t0 = 0; t0 < nl; t0 += GT) {
                const int k = t0 + threadIdx.x;
                if (k < nl) {
                    float4 qh, ql;
                    float gm;
                    if (pass == 0) {
                        const int j = E[k];
                        qh = xh[j];
                        ql = xl[j];
                        gm = (float)(G * m[j] * gscale);
                    } else {
                        const int cc = S[k];
                        qh = ch[cc];
                        ql = cl[cc];
                        gm = qh.w;
                    }
                    tile[threadIdx.x] = make_float4(df_diff(qh.x, ql.x, c_h.x, c_l.x), df_diff(qh.y, ql.y, c_h.y, c_l.y),
                                                    df_diff(qh.z, ql.z, c_h.z, c_l.z), gm);
                }
                __syncthreads();
                const int tn = min(GT, nl - t0);
                float P0 = 0.f, P1 = 0.f, P2 = 0.f, P3 = 0.f;
                for (int t = 0; t < tn; ++t) {
                    const float4 q = tile[t];
                    const float dx = xi - q.x, dy = yi - q.y, dz = zi - q.z;
                    const float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, eps2)));
                    const float ri = rsqrt_a(r2);
                    const float mri = q.w * ri;
                    const float mr3 = mri * ri * ri;
                    P0 = fmaf(-mr3, dx, P0);
                    P1 = fmaf(-mr3, dy, P1);
                    P2 = fmaf(-mr3, dz, P2);
                    P3 -= mri;
                }
                D[0] += (double)P0;
                D[1] += (double)P1;
                D[2] += (double)P2;
                D[3] += (double)P3;
                __syncthreads();
            }
        }
        if (act) {
            gx[i] = D[0] * inv_gscale;
            gy[i] = D[1] * inv_gscale;
            gz[i] = D[2] * inv_gscale;
            pot[i] = D[3] * inv_gscale;
        }
    }
}

// ---------------------------------------------------------------------------
// Mixed-precision tree gravity with the walk fused in: one CTA per i-group.
// All warps walk the octree breadth-first together, T / 4 opened cells per
// iteration (four lanes per cell, two children per lane), with the opening
// rule and append order of k_grav_lists / or_grav_walk, into shared-memory EPJ
// and SPJ buffers; when the buffers are full, or the walk has ended, every
// thread accumulates the buffered interactions.  No interaction list reaches
// global memory.  The queue holds whole cell records (first child, children |
// level << 8, start, count), loaded together with the child's centre of mass
// when the child is tested, so an iteration waits on one global load.
//
// Accumulation: each thread carries two i-particles (ii and ii + Wt, Wt =
// roundup(count / 2, 8)), and the block's P = T / Wt copies of the group
// split each tile of j between them, four consecutive j per round in paired
// FP32 arithmetic; small groups keep the FP32 lanes busy and every
// shared-memory read feeds two interactions.
//
// Two block shapes (T threads): 128 threads with a ring of 1,024 cell records,
// eight blocks per SM, the one launched; 256 threads with 2,048 records, four
// blocks per SM, relaunched for the whole pass when a walk's breadth-first
// front outgrows the smaller ring (opening angles near 0 on large bodies).  The
// widest front of the 1M and 4M impacts at theta 0.5 is 456 records.  Measured
// at 1M (kernel time), 128 threads: eight blocks per SM 1.75 ms; seven (no
// spills) 1.82 ms; nine or ten (56 / 48 registers, smaller buffers and tiles,
// more spills) 1.80 / 2.65 ms; six with 1,024-entry buffers 1.83 ms; five with
// the 2,048 ring 1.94 ms.  256 threads, four per SM: 1.94 ms (buffers of 2,048
// and tiles of 256 1.96 ms, 1,024 and 1,024 2.09 ms, 2,048 and 1,024 at three
// blocks per SM 2.00 ms).  More independent blocks let one block's walk
// overlap another's sums.
template <int T>
struct GravShape;
template <>
struct GravShape<128> {
    static constexpr int Q = 1024;     // BFS ring of opened cell records (power of two)
    static constexpr int E = 768;      // buffered EPJ particle indices
    static constexpr int S = 768;      // buffered SPJ cell indices
    static constexpr int TILE = 256;   // j entries per shared-memory tile (TILE / T staged per thread)
    static constexpr int MIN_BLOCKS = 8;
};
template <>
struct GravShape<256> {
    static constexpr int Q = 2048;
    static constexpr int E = 1536;
    static constexpr int S = 1536;
    static constexpr int TILE = 512;
    static constexpr int MIN_BLOCKS = 4;
};

__device__ __forceinline__ void grav_acc(float px, float py, float pz, float e2, float4 q, float &a0, float &a1,
                                         float &a2, float &a3) {
    const float dx = px - q.x, dy = py - q.y, dz = pz - q.z;
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, e2)));
    const float ri = rsqrt_a(r2);
    const float mri = q.w * ri;
    const float mr3 = mri * ri * ri;
    a0 = fmaf(-mr3, dx, a0);
    a1 = fmaf(-mr3, dy, a1);
    a2 = fmaf(-mr3, dz, a2);
    a3 -= mri;
}

// grav_acc for two j at once (x, y, z, m: the pair's coordinates relative to the group origin and
// masses), with the i-particle's negated coordinates and softening paired with themselves.  Per
// interaction the same operations and roundings as grav_acc (q - p = -(p - q) exactly); the two j
// accumulate in the two halves of a0..a3, and a3 sums +m / r (the potential's negative).
__device__ __forceinline__ void grav_acc2(f32x2 nx, f32x2 ny, f32x2 nz, f32x2 e2, f32x2 x, f32x2 y, f32x2 z,
                                          f32x2 m, f32x2 &a0, f32x2 &a1, f32x2 &a2, f32x2 &a3) {
    const f32x2 dx = f2_add(x, nx), dy = f2_add(y, ny), dz = f2_add(z, nz);
    const f32x2 r2 = f2_fma(dx, dx, f2_fma(dy, dy, f2_fma(dz, dz, e2)));
    float ra, rb;
    f2_unpack(r2, ra, rb);
    const f32x2 ri = f2_pack(rsqrt_a(ra), rsqrt_a(rb));
    const f32x2 mri = f2_mul(m, ri);
    const f32x2 mr3 = f2_mul(f2_mul(mri, ri), ri);
    a0 = f2_fma(mr3, dx, a0);
    a1 = f2_fma(mr3, dy, a1);
    a2 = f2_fma(mr3, dz, a2);
    a3 = f2_add(a3, mri);
}

template <int GF_T>
__global__ void __launch_bounds__(GF_T, GravShape<GF_T>::MIN_BLOCKS)
k_grav_fused32(const int *__restrict__ group_cell, const int4 *__restrict__ cinfo, const double4 *__restrict__ com,
               const double *__restrict__ rb_all, const int *__restrict__ prun, const double *__restrict__ x,
               const double *__restrict__ y,
               const double *__restrict__ z, const float4 *__restrict__ xh, const float4 *__restrict__ xl,
               const double *__restrict__ h, const float4 *__restrict__ ch, const float4 *__restrict__ cl, float gms,
               double *gx, double *gy, double *gz, double *pot, int *n_epj, int *n_spj, int *err) {
    constexpr int GF_Q = GravShape<GF_T>::Q, GF_E = GravShape<GF_T>::E, GF_S = GravShape<GF_T>::S;
    constexpr int GF_TILE = GravShape<GF_T>::TILE, GF_W = GF_T / 32;
    static_assert(GF_TILE % GF_T == 0, "tile: whole loads per thread");
    static_assert(4 * GF_TILE * 4 >= GF_T * 4 * 8 || GF_E * 4 >= GF_T * 4 * 8, "room for the partition reduction");
    __shared__ int4 s_q[GF_Q];
    __shared__ __align__(16) int s_e[GF_E];
    __shared__ int s_s[GF_S];
    // the j tile as four arrays, so a thread's four consecutive entries load as two packed pairs;
    // also the reduction buffer of the partitions
    __shared__ __align__(16) float s_tile[4][GF_TILE];
    float *s_tx = s_tile[0], *s_ty = s_tile[1], *s_tz = s_tile[2], *s_tm = s_tile[3];
    __shared__ int s_w[2][GF_W][3];            // per warp: leaf particles, far children, near children
    __shared__ double s_rb[MAX_LEVELS];
    __shared__ float s_rbf[MAX_LEVELS];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned below = (1u << lane) - 1u;
    const int4 gi = cinfo[group_cell[blockIdx.x]];
    const int s = gi.z, cnt_all = gi.w;
    const float4 c_h = xh[s], c_l = xl[s];     // group origin: its first particle
    const int root = prun[s];                  // the group's run: its octree root and opening radii
    const double *rb = rb_all + (int64_t)root * RB_STRIDE;
    for (int l = tid; l < MAX_LEVELS; l += GF_T) {
        s_rb[l] = rb[8 + l];
        s_rbf[l] = (float)rb[8 + l];
    }
    // bounding box of the whole group
    // (one warp: the FP64 min / max and their shuffles are slow on this GPU's FP64 pipe)
    __shared__ double s_gbox[6];   // the group's box in FP64, for the exact opening test
    if (warp == 0) {
        double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int k = lane; k < cnt_all; k += 32) {
            const double p[3] = {x[s + k], y[s + k], z[s + k]};
            for (int d = 0; d < 3; ++d) {
                lo[d] = fmin(lo[d], p[d]);
                hi[d] = fmax(hi[d], p[d]);
            }
        }
        for (int d = 0; d < 3; ++d)
            for (int o = 16; o > 0; o >>= 1) {
                lo[d] = fmin(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
                hi[d] = fmax(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
            }
        if (lane == 0)
            for (int d = 0; d < 3; ++d) {
                s_gbox[d] = lo[d];
                s_gbox[3 + d] = hi[d];
            }
    }
    __syncthreads();
    // the box relative to the group origin, in FP32, for the fast opening test
    float lof[3], hif[3];
    {
        const float oh[3] = {c_h.x, c_h.y, c_h.z}, ol[3] = {c_l.x, c_l.y, c_l.z};
        for (int d = 0; d < 3; ++d) {
            const double o = (double)oh[d] + (double)ol[d];
            lof[d] = (float)(s_gbox[d] - o);
            hif[d] = (float)(s_gbox[3 + d] - o);
        }
    }
    // walk lanes: 64 opened cells per iteration, four lanes per cell, two children per lane
    // (octants k and k + 4); appends go cell by cell, first children before second children
    const int q = tid >> 2, k = tid & 3, qw = lane >> 2;
    const unsigned cellm = 0xFu << (qw * 4), before = (1u << (qw * 4)) - 1u;
    int tot_e = 0, tot_s = 0;
    for (int i_base = 0; i_base < cnt_all; i_base += 2 * GF_T) {
        const int cnt = min(2 * GF_T, cnt_all - i_base);
        // partitions of ceil(cnt / 2) lanes, rounded up to 8 lanes below 16 (a warp then holds at most
        // four partitions, whose tile reads take as many shared-memory wavefronts); at 1M, 88% of the
        // slots carry an i-particle (86% with every width rounded up to 8: 1.76 -> 1.73 ms)
        const int half = (cnt + 1) / 2;
        const int Wt = half >= 16 ? half : (half + 7) & ~7, P = GF_T / Wt;
        const int TE = GF_TILE / (4 * P) * (4 * P);   // tile entries: a multiple of every partition's stride
        const int part = tid / Wt, ii = tid - part * Wt;
        const bool slot = part < P;
        float px[2], py[2], pz[2], e2[2];
        for (int u = 0; u < 2; ++u) {
            const int iu = ii + u * Wt;
            px[u] = py[u] = pz[u] = 0.f;
            e2[u] = 1.f;
            if (slot && iu < cnt) {
                const int i = s + i_base + iu;
                const float4 ph = xh[i], pl = xl[i];
                px[u] = df_diff(ph.x, pl.x, c_h.x, c_l.x);
                py[u] = df_diff(ph.y, pl.y, c_h.y, c_l.y);
                pz[u] = df_diff(ph.z, pl.z, c_h.z, c_l.z);
                const double hh = h[i];
                e2[u] = (float)(hh * hh);
            }
        }
        float Dh[2][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}}, Dl[2][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}};
        int head = 0, tail = 1, it = 0;
        if (tid == 0) s_q[0] = cinfo[root];   // the run's root, level 0
        __syncthreads();
        for (;;) {
            // ---- walk until the buffers are full or the queue is empty
            int ne = 0, ns = 0, done = 0;
            for (;; ++it) {
                if (head >= tail) {
                    done = 1;
                    break;
                }
                const int nproc = min(GF_T / 4, tail - head);
                const bool a = q < nproc;
                const int4 ci = a ? s_q[(head + q) & (GF_Q - 1)] : make_int4(0, 0, 0, 0);
                const int nch = ci.y & 255, lev = ci.y >> 8;
                const bool leaf = a && nch == 0;
                const int lc = leaf ? ci.w : 0;   // same in the four lanes of a cell
                bool near[2] = {false, false}, far[2] = {false, false};
                int chc[2] = {0, 0};
                int4 crec[2] = {make_int4(0, 0, 0, 0), make_int4(0, 0, 0, 0)};
#pragma unroll
                for (int hh = 0; hh < 2; ++hh) {
                    const int kk = k + 4 * hh;
                    if (!(a && kk < nch)) continue;
                    chc[hh] = ci.x + kk;
                    const float4 qh = ch[chc[hh]], ql = cl[chc[hh]];
                    crec[hh] = cinfo[chc[hh]];
                    const float rbf = s_rbf[lev + 1];
                    // FP32 distance from the box on coordinates relative to the group origin, with a
                    // bound on its error; inside the bound the FP64 test of the list walk decides
                    const float pr[3] = {df_diff(qh.x, ql.x, c_h.x, c_l.x), df_diff(qh.y, ql.y, c_h.y, c_l.y),
                                         df_diff(qh.z, ql.z, c_h.z, c_l.z)};
                    const float pa[3] = {fabsf(qh.x) + fabsf(c_h.x), fabsf(qh.y) + fabsf(c_h.y),
                                         fabsf(qh.z) + fabsf(c_h.z)};
                    float d2f = 0.0f, E = 0.0f;
                    for (int d = 0; d < 3; ++d) {
                        const float b = pr[d] < lof[d] ? lof[d] : (pr[d] > hif[d] ? hif[d] : pr[d]);
                        const float dd = fabsf(b - pr[d]);
                        const float ed = 2.384185791015625e-07f * (fabsf(pr[d]) + fabsf(b) + dd) +
                                         2.842170943040401e-14f * pa[d];   // 2^-22 relative, 2^-45 absolute
                        d2f = fmaf(dd, dd, d2f);
                        E = fmaf(2.0f * dd + ed, ed, E);
                    }
                    E += 4.76837158203125e-07f * (d2f + rbf);   // 2^-21: sums and the rounding of rb
                    bool nr;
                    if (fabsf(d2f - rbf) > E) {
                        nr = d2f <= rbf;
                    } else {
                        const double4 cm = com[chc[hh]];
                        const double pp[3] = {cm.x, cm.y, cm.z};
                        double dd[3];
                        for (int d = 0; d < 3; ++d) {
                            const double l = s_gbox[d], u = s_gbox[3 + d];
                            dd[d] = (pp[d] < l) ? __dsub_rn(l, pp[d]) : ((pp[d] > u) ? __dsub_rn(pp[d], u) : 0.0);
                        }
                        const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dd[0], dd[0]), __dmul_rn(dd[1], dd[1])),
                                                    __dmul_rn(dd[2], dd[2]));
                        nr = d2 <= s_rb[lev + 1];
                    }
                    near[hh] = nr;
                    far[hh] = !nr;
                }
                const unsigned nm0 = __ballot_sync(0xffffffffu, near[0]), nm1 = __ballot_sync(0xffffffffu, near[1]);
                const unsigned fm0 = __ballot_sync(0xffffffffu, far[0]), fm1 = __ballot_sync(0xffffffffu, far[1]);
                int lpre = 0, lsum = 0;
                for (int g = 0; g < 8; ++g) {
                    const int v = __shfl_sync(0xffffffffu, lc, g * 4);
                    lpre += g < qw ? v : 0;
                    lsum += v;
                }
                const int buf = it & 1;
                if (lane == 0) {
                    s_w[buf][warp][0] = lsum;
                    s_w[buf][warp][1] = __popc(fm0) + __popc(fm1);
                    s_w[buf][warp][2] = __popc(nm0) + __popc(nm1);
                }
                __syncthreads();
                int oe = 0, of = 0, on = 0, te = 0, tf = 0, tn = 0;
                for (int w = 0; w < GF_W; ++w) {
                    const int e0 = s_w[buf][w][0], f0 = s_w[buf][w][1], n0 = s_w[buf][w][2];
                    if (w < warp) {
                        oe += e0;
                        of += f0;
                        on += n0;
                    }
                    te += e0;
                    tf += f0;
                    tn += n0;
                }
                if (ne + te > GF_E || ns + tf > GF_S) {   // flush first, then redo this batch
                    if (ne == 0 && ns == 0) {              // a batch larger than the buffers: give up
                        if (tid == 0) atomicOr(err, ERR_GRAV_OVERFLOW);
                        done = 1;
                    }
                    ++it;
                    break;
                }
                if (tail - head - nproc + tn > GF_Q) {
                    if (tid == 0) atomicOr(err, ERR_GRAV_OVERFLOW);
                    done = 1;
                    ++it;
                    break;
                }
                if (leaf)
                    for (int t = k; t < lc; t += 4) s_e[ne + oe + lpre + t] = ci.z + t;
                {
                    // order within the warp: cell by cell, a cell's first children, then its second
                    const int f_pre = __popc(fm0 & before) + __popc(fm1 & before);
                    const int n_pre = __popc(nm0 & before) + __popc(nm1 & before);
                    const int f_pos[2] = {f_pre + __popc(fm0 & cellm & below),
                                          f_pre + __popc(fm0 & cellm) + __popc(fm1 & cellm & below)};
                    const int n_pos[2] = {n_pre + __popc(nm0 & cellm & below),
                                          n_pre + __popc(nm0 & cellm) + __popc(nm1 & cellm & below)};
#pragma unroll
                    for (int hh = 0; hh < 2; ++hh) {
                        if (far[hh]) s_s[ns + of + f_pos[hh]] = chc[hh];
                        if (near[hh]) {
                            int4 r = crec[hh];
                            r.y = (r.y & 255) | ((lev + 1) << 8);
                            s_q[(tail + on + n_pos[hh]) & (GF_Q - 1)] = r;
                        }
                    }
                }
                ne += te;
                ns += tf;
                head += nproc;
                tail += tn;
                __syncthreads();   // the records and buffer entries written above
            }
            if (i_base == 0) {
                tot_e += ne;
                tot_s += ns;
            }
            // ---- accumulate the buffered EPJ, then SPJ
            for (int pass = 0; pass < 2; ++pass) {
                const int nl = pass == 0 ? ne : ns;
                for (int t0 = 0; t0 < nl; t0 += TE) {
#pragma unroll
                    for (int r = 0; r < GF_TILE / GF_T; ++r) {
                        const int e = tid + r * GF_T, kk = t0 + e;
                        float4 v = make_float4(0.f, 0.f, 0.f, 0.f);   // zero mass pads the tile
                        if (e < TE && kk < nl) {
                            float4 qh, ql;
                            float gm;
                            if (pass == 0) {
                                const int j = s_e[kk];
                                qh = xh[j];
                                ql = xl[j];
                                gm = qh.w * gms;
                            } else {
                                const int cc = s_s[kk];
                                qh = ch[cc];
                                ql = cl[cc];
                                gm = qh.w;
                            }
                            v = make_float4(df_diff(qh.x, ql.x, c_h.x, c_l.x), df_diff(qh.y, ql.y, c_h.y, c_l.y),
                                            df_diff(qh.z, ql.z, c_h.z, c_l.z), gm);
                        }
                        s_tx[e] = v.x;
                        s_ty[e] = v.y;
                        s_tz[e] = v.z;
                        s_tm[e] = v.w;
                    }
                    __syncthreads();
                    if (slot) {
                        const int step = 4 * P;
                        const int tnr = (min(TE, nl - t0) + step - 1) / step * step;   // <= TE: step divides it
                        f32x2 A[2][4] = {{0ull, 0ull, 0ull, 0ull}, {0ull, 0ull, 0ull, 0ull}};
                        for (int t = 4 * part; t < tnr; t += step) {
                            const ulonglong2 X = *reinterpret_cast<const ulonglong2 *>(s_tx + t);
                            const ulonglong2 Y = *reinterpret_cast<const ulonglong2 *>(s_ty + t);
                            const ulonglong2 Z = *reinterpret_cast<const ulonglong2 *>(s_tz + t);
                            const ulonglong2 M = *reinterpret_cast<const ulonglong2 *>(s_tm + t);
#pragma unroll
                            for (int u = 0; u < 2; ++u) {
                                const f32x2 nx = f2_pack(-px[u], -px[u]), ny = f2_pack(-py[u], -py[u]),
                                            nz = f2_pack(-pz[u], -pz[u]), ee = f2_pack(e2[u], e2[u]);
                                grav_acc2(nx, ny, nz, ee, X.x, Y.x, Z.x, M.x, A[u][0], A[u][1], A[u][2], A[u][3]);
                                grav_acc2(nx, ny, nz, ee, X.y, Y.y, Z.y, M.y, A[u][0], A[u][1], A[u][2], A[u][3]);
                            }
                        }
#pragma unroll
                        for (int u = 0; u < 2; ++u)
                            for (int c4 = 0; c4 < 4; ++c4) {
                                float lo, hi;
                                f2_unpack(A[u][c4], lo, hi);
                                df_add(Dh[u][c4], Dl[u][c4], c4 == 3 ? -(lo + hi) : lo + hi);
                            }
                    }
                    __syncthreads();
                }
            }
            if (done) break;
        }
        // ---- sum the partitions of each i-particle
        // GF_T x 4 doubles, in the tile or the EPJ buffer (whichever holds them; both are free here)
        double *red = 4 * GF_TILE * 4 >= GF_T * 4 * 8 ? reinterpret_cast<double *>(&s_tile[0][0])
                                                       : reinterpret_cast<double *>(s_e);
        for (int u = 0; u < 2; ++u) {
            for (int c4 = 0; c4 < 4; ++c4) red[c4 * GF_T + tid] = (double)Dh[u][c4] + (double)Dl[u][c4];
            __syncthreads();
            const int iu = ii + u * Wt;
            if (slot && part == 0 && iu < cnt) {
                double r[4] = {0, 0, 0, 0};
                for (int p2 = 0; p2 < P; ++p2)
                    for (int c4 = 0; c4 < 4; ++c4) r[c4] += red[c4 * GF_T + p2 * Wt + ii];
                const int i = s + i_base + iu;
                gx[i] = r[0];
                gy[i] = r[1];
                gz[i] = r[2];
                pot[i] = r[3];
            }
            __syncthreads();
        }
    }
    if (tid == 0) {
        n_epj[blockIdx.x] = tot_e;   // of the first chunk of i when a group has more than 512 particles
        n_spj[blockIdx.x] = tot_s;
    }
}

// ---------------------------------------------------------------------------
// integrator (class.h:201-229), external damping (GI.h:458-465), dt (integral.h:4-20)

struct IntegArgs {
    double *x, *y, *z, *vx, *vy, *vz, *ax, *ay, *az, *gx, *gy, *gz, *vhx, *vhy, *vhz, *u, *ud, *uh;
    const int *prun;        // run of each particle
    const double *run_dt;   // dt of the step, per run
};

__global__ void k_kick_drift_predict(int n, IntegArgs a) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double dt = a.run_dt[a.prun[i]];
    const double ax = a.ax[i] + a.gx[i], ay = a.ay[i] + a.gy[i], az = a.az[i] + a.gz[i];
    const double hx = a.vx[i] + 0.5 * dt * ax, hy = a.vy[i] + 0.5 * dt * ay, hz = a.vz[i] + 0.5 * dt * az;
    a.vhx[i] = hx;
    a.vhy[i] = hy;
    a.vhz[i] = hz;
    a.uh[i] = a.u[i] + 0.5 * dt * a.ud[i];
    a.x[i] += dt * hx;
    a.y[i] += dt * hy;
    a.z[i] += dt * hz;
    a.vx[i] += dt * ax;
    a.vy[i] += dt * ay;
    a.vz[i] += dt * az;
    a.u[i] += dt * a.ud[i];
}

__global__ void k_final_kick(int n, IntegArgs a, double damp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double dt = a.run_dt[a.prun[i]];
    if (dt == 0.0) damp = 1.0;   // a run's prologue step (dampMotion belongs to the loop body, main.cpp:152)
    a.vx[i] = (a.vhx[i] + 0.5 * dt * (a.ax[i] + a.gx[i])) * damp;
    a.vy[i] = (a.vhy[i] + 0.5 * dt * (a.ay[i] + a.gy[i])) * damp;
    a.vz[i] = (a.vhz[i] + 0.5 * dt * (a.az[i] + a.gz[i])) * damp;
    a.u[i] = a.uh[i] + 0.5 * dt * a.ud[i];
}

__global__ void k_ext_force(int n, IntegArgs a, const double *dt, const unsigned char *run_damp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !run_damp[a.prun[i]]) return;
    const double d = dt[i];
    a.ax[i] += -a.vx[i] * 0.05 / d;
    a.ay[i] += -a.vy[i] * 0.05 / d;
    a.az[i] += -a.vz[i] * 0.05 / d;
}

constexpr int RED_BLOCKS = 304;

__global__ void k_min_partial(int n, const double *v, double *part) {
    double r = 1.0e30;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double d = v[i];
        r = (d < r) ? d : r;   // std::min(r, d) with r first, integral.h:16
        if (d != d) r = d;     // a NaN dt propagates so the host sees it
    }
    for (int o = 16; o > 0; o >>= 1) {
        const double t = __shfl_xor_sync(0xffffffffu, r, o);
        r = (t < r || t != t) ? t : r;
    }
    __shared__ double s[32];
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = r;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) r = (s[w] < r || s[w] != s[w]) ? s[w] : r;
        part[blockIdx.x] = r;
    }
}

__global__ void k_min_final(const double *part, int nb, double *out) {
    double r = 1.0e30;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) r = (part[b] < r || part[b] != part[b]) ? part[b] : r;
    for (int o = 16; o > 0; o >>= 1) {
        const double t = __shfl_xor_sync(0xffffffffu, r, o);
        r = (t < r || t != t) ? t : r;
    }
    __shared__ double s[32];
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = r;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) r = (s[w] < r || s[w] != s[w]) ? s[w] : r;
        *out = r;
    }
}

// per run: one block per tile (tiles aligned to run starts), then one block per run over its tiles
__device__ double block_min(double r) {
    for (int o = 16; o > 0; o >>= 1) {
        const double t = __shfl_xor_sync(0xffffffffu, r, o);
        r = (t < r || t != t) ? t : r;
    }
    __shared__ double s[32];
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = r;
    __syncthreads();
    if (threadIdx.x == 0)
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) r = (s[w] < r || s[w] != s[w]) ? s[w] : r;
    return r;
}

__global__ void k_min_tiles(const double *v, const int4 *tiles, double *part) {
    const int4 t = tiles[blockIdx.x];
    double r = 1.0e30;
    for (int i = t.x + threadIdx.x; i < t.x + t.y; i += blockDim.x) {
        const double d = v[i];
        r = (d < r) ? d : r;   // std::min(r, d) with r first, integral.h:16
        if (d != d) r = d;     // a NaN dt propagates so the host sees it
    }
    r = block_min(r);
    if (threadIdx.x == 0) part[blockIdx.x] = r;
}

__global__ void k_min_runs(const double *part, const int4 *info, double *out) {
    const int4 q = info[blockIdx.x];
    double r = 1.0e30;
    for (int b = q.z + threadIdx.x; b < q.z + q.w; b += blockDim.x) r = (part[b] < r || part[b] != part[b]) ? part[b] : r;
    r = block_min(r);
    if (threadIdx.x == 0) out[blockIdx.x] = r;
}

// conserved quantities, fixed-order two-stage reduction in FP64
__global__ void k_diag_partial(int n, const double *x, const double *y, const double *z, const double *vx,
                               const double *vy, const double *vz, const double *m, const double *u,
                               const double *pot, double *part) {
    double q[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double mi = m[i];
        const double v2 = vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i];
        q[0] += mi * (u[i] + 0.5 * v2 + 0.5 * pot[i]);
        q[1] += mi * vx[i];
        q[2] += mi * vy[i];
        q[3] += mi * vz[i];
        q[4] += mi * (y[i] * vz[i] - z[i] * vy[i]);
        q[5] += mi * (z[i] * vx[i] - x[i] * vz[i]);
        q[6] += mi * (x[i] * vy[i] - y[i] * vx[i]);
        q[7] += mi;
    }
    __shared__ double s[8][32];
    for (int k = 0; k < 8; ++k) {
        double v = q[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) s[k][threadIdx.x >> 5] = v;
    }
    __syncthreads();
    if (threadIdx.x < 8) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += s[threadIdx.x][w];
        part[blockIdx.x * 8 + threadIdx.x] = v;
    }
}

// per run: tiles (k_diag_partial over one tile's range), then each run's tiles in order
__global__ void k_diag_tiles(const double *x, const double *y, const double *z, const double *vx, const double *vy,
                             const double *vz, const double *m, const double *u, const double *pot, const int4 *tiles,
                             double *part) {
    const int4 t = tiles[blockIdx.x];
    double q[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = t.x + threadIdx.x; i < t.x + t.y; i += blockDim.x) {
        const double mi = m[i];
        const double v2 = vx[i] * vx[i] + vy[i] * vy[i] + vz[i] * vz[i];
        q[0] += mi * (u[i] + 0.5 * v2 + 0.5 * pot[i]);
        q[1] += mi * vx[i];
        q[2] += mi * vy[i];
        q[3] += mi * vz[i];
        q[4] += mi * (y[i] * vz[i] - z[i] * vy[i]);
        q[5] += mi * (z[i] * vx[i] - x[i] * vz[i]);
        q[6] += mi * (x[i] * vy[i] - y[i] * vx[i]);
        q[7] += mi;
    }
    __shared__ double s[8][32];
    for (int k = 0; k < 8; ++k) {
        double v = q[k];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) s[k][threadIdx.x >> 5] = v;
    }
    __syncthreads();
    if (threadIdx.x < 8) {
        double v = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) v += s[threadIdx.x][w];
        part[blockIdx.x * 8 + threadIdx.x] = v;
    }
}

__global__ void k_diag_runs(const double *part, const int4 *info, int R, double *out) {
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < R * 8; k += gridDim.x * blockDim.x) {
        const int r = k >> 3, c = k & 7;
        const int4 q = info[r];
        double v = 0.0;
        for (int b = q.z; b < q.z + q.w; ++b) v += part[b * 8 + c];
        out[k] = v;
    }
}

__global__ void k_diag_final(const double *part, int nb, double *out) {
    if (threadIdx.x < 8 && blockIdx.x == 0) {
        double v = 0.0;
        for (int b = 0; b < nb; ++b) v += part[b * 8 + threadIdx.x];
        out[threadIdx.x] = v;
    }
}

__global__ void k_init_smth(int n, const double *m, const double *dens, double *h, double *gradh) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    h[i] = SMTH_COEF * pow(m[i] / dens[i], 1.0 / 3.0);
    gradh[i] = 1.0;
}

__global__ void k_sum_cnt(int n, const int *cnt, unsigned long long *out) {
    unsigned long long v = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v += (unsigned)cnt[i];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, v);
}

__global__ void k_sum_grav_pairs(int ng, const int *group_cell, const int *count, const int *ne, const int *ns,
                                 unsigned long long *out) {
    unsigned long long v = 0;
    for (int g = blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += gridDim.x * blockDim.x)
        v += (unsigned long long)count[group_cell[g]] * (unsigned long long)(ne[g] + ns[g]);
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(out, v);
}

}  // namespace sph

using namespace sph;

#define CF(f) FLD(ctx->F, f, ctx->cap)

static IntegArgs integ_args(sph_ctx *ctx) {
    return IntegArgs{CF(SPH_X),  CF(SPH_Y),  CF(SPH_Z),  CF(SPH_VX),  CF(SPH_VY),  CF(SPH_VZ),
                     CF(SPH_AX), CF(SPH_AY), CF(SPH_AZ), CF(SPH_GX),  CF(SPH_GY),  CF(SPH_GZ),
                     CF(SPH_VHX), CF(SPH_VHY), CF(SPH_VHZ), CF(SPH_ENG), CF(SPH_ENGDOT), CF(SPH_ENGHALF),
                     ctx->runs.prun, ctx->runs.dt_dev};
}

static int ensure_mixed_buffers(sph_ctx *ctx) {
    if (ctx->xh) return SPH_OK;
    const size_t b = sizeof(float4) * (size_t)ctx->cap;
    float4 **bufs[] = {&ctx->xh, &ctx->xl, &ctx->vhf, &ctx->vlf};
    for (auto p : bufs)
        if (cudaMalloc((void **)p, b) != cudaSuccess) {
            cudaGetLastError();
            return sph_fail(ctx, SPH_ERR_OOM, "mixed-precision buffers");
        }
    return SPH_OK;
}

int sph_pack_mixed(sph_ctx *ctx) {
    SPH_TRY(ensure_mixed_buffers(ctx));
    const int n = (int)ctx->n;
    k_pack_df<<<sph_div_up(n, 256), 256, 0, ctx->stream>>>(n, CF(SPH_X), CF(SPH_Y), CF(SPH_Z), CF(SPH_VX), CF(SPH_VY),
                                                           CF(SPH_VZ), CF(SPH_MASS), CF(SPH_SMTH),
                                                           ctx->mscale, ctx->xh, ctx->xl, ctx->vhf,
                                                           ctx->vlf); ++ctx->launches;
    SPH_CUDA(ctx, cudaGetLastError());
    return SPH_OK;
}

int sph_pass_density(sph_ctx *ctx, int build_lists) {
    if (build_lists) SPH_TRY(sph_build_sph_lists(ctx, 0));
    const int n = (int)ctx->n;
    const SphLists &L = ctx->lists[0];
    if (ctx->cfg.precision == SPH_PREC_MIXED) {
        k_density32<<<sph_div_up(n, PT), PT, 0, ctx->stream>>>(n, ctx->xh, ctx->xl, CF(SPH_MASS), CF(SPH_SMTH),
                                                              CF(SPH_DENS), L.nbr, L.cnt, ctx->sup.map(),
                                                              (float)(WNORM / (PI_D * ctx->mscale))); ++ctx->launches;
    } else {
        k_density64<<<sph_div_up(n, PT), PT, 0, ctx->stream>>>(n, CF(SPH_X), CF(SPH_Y), CF(SPH_Z), CF(SPH_MASS),
                                                              CF(SPH_SMTH), CF(SPH_DENS), L.nbr, L.cnt, ctx->sup.map()); ++ctx->launches;
    }
    SPH_CUDA(ctx, cudaGetLastError());
    return sph_nbr_refresh_h(ctx);
}

int sph_pass_eos(sph_ctx *ctx) {
    const int n = (int)ctx->n;
    k_eos<<<sph_div_up(n, PT), PT, 0, ctx->stream>>>(n, ctx->mats_dev, ctx->mat, CF(SPH_DENS), CF(SPH_ENG),
                                                    CF(SPH_PRES), CF(SPH_SNDS)); ++ctx->launches;
    SPH_CUDA(ctx, cudaGetLastError());
    return SPH_OK;
}

int sph_pass_derivative(sph_ctx *ctx, int build_lists) {
    if (build_lists) SPH_TRY(sph_build_sph_lists(ctx, 0));
    const int n = (int)ctx->n;
    const SphLists &L = ctx->lists[0];
    if (ctx->cfg.precision == SPH_PREC_MIXED) {
        DrvtArgs32 a{ctx->xh,     ctx->xl,      ctx->vhf,     ctx->vlf,      CF(SPH_SMTH), CF(SPH_DENS),
                     CF(SPH_SNDS), CF(SPH_DIVV), CF(SPH_ROTX), CF(SPH_ROTY),  CF(SPH_ROTZ), CF(SPH_GRADH),
                     CF(SPH_BAL),  L.nbr,        L.cnt,        ctx->sup.map(),
                     (float)(WNORM / (PI_D * ctx->mscale))};
        // threads per i-particle: chosen by sph_autotune (1 unless tuned)
        const int tpi = ctx->tune.drvt_tpi;
        auto kd = tpi == 4 ? k_drvt32<4> : (tpi == 2 ? k_drvt32<2> : k_drvt32<1>);
        kd<<<sph_div_up((int64_t)n * tpi, PT), PT, 0, ctx->stream>>>(n, a); ++ctx->launches;
    } else {
        DrvtArgs a{CF(SPH_X),    CF(SPH_Y),    CF(SPH_Z),    CF(SPH_VX),    CF(SPH_VY),   CF(SPH_VZ),
                   CF(SPH_MASS), CF(SPH_SMTH), CF(SPH_DENS), CF(SPH_SNDS),  CF(SPH_DIVV), CF(SPH_ROTX),
                   CF(SPH_ROTY), CF(SPH_ROTZ), CF(SPH_GRADH), CF(SPH_BAL), L.nbr,        L.cnt,
                   ctx->sup.map()};
        k_drvt64<<<sph_div_up(n, PT), PT, 0, ctx->stream>>>(n, a); ++ctx->launches;
    }
    SPH_CUDA(ctx, cudaGetLastError());
    return SPH_OK;
}

int sph_pass_hydro(sph_ctx *ctx, int build_lists) {
    if (build_lists) SPH_TRY(sph_build_sph_lists(ctx, 1));
    const int n = (int)ctx->n;
    const SphLists &L = ctx->lists[1];
    // scratch: 2 x float4 or 1 x double4 per particle, in the F2 ping-pong block (free between sorts)
    if (ctx->cfg.precision == SPH_PREC_MIXED) {
        float4 *hA = (float4 *)ctx->F2;
        k_hydro_pack32<<<sph_div_up(n, 256), 256, 0, ctx->stream>>>(n, CF(SPH_SMTH), CF(SPH_DENS), CF(SPH_PRES),
                                                                    CF(SPH_SNDS), CF(SPH_GRADH), CF(SPH_BAL), hA,
                                                                    ctx->xl, ctx->vhf, ctx->vlf); ++ctx->launches;
        HydroArgs32 a{ctx->xh,    ctx->xl,    ctx->vhf,   ctx->vlf,       hA,    CF(SPH_SMTH),
                      CF(SPH_AX), CF(SPH_AY), CF(SPH_AZ), CF(SPH_ENGDOT), CF(SPH_DT), L.nbr, L.cnt,
                      ctx->sup.map(),    (float)(WNORM / (PI_D * ctx->mscale))};
        const int tpi = ctx->tune.hydro_tpi;
        auto kh = tpi == 4 ? k_hydro32<4> : (tpi == 2 ? k_hydro32<2> : k_hydro32<1>);
        kh<<<sph_div_up((int64_t)n * tpi, PT), PT, 0, ctx->stream>>>(n, a); ++ctx->launches;
    } else {
        double4 *aux = (double4 *)ctx->F2;
        k_hydro_aux64<<<sph_div_up(n, 256), 256, 0, ctx->stream>>>(n, CF(SPH_SMTH), CF(SPH_DENS), CF(SPH_PRES),
                                                                   CF(SPH_GRADH), aux); ++ctx->launches;
        HydroArgs a{CF(SPH_X),    CF(SPH_Y),    CF(SPH_Z),     CF(SPH_VX),   CF(SPH_VY),  CF(SPH_VZ),
                    CF(SPH_MASS), CF(SPH_SMTH), CF(SPH_DENS),  CF(SPH_PRES), CF(SPH_SNDS), CF(SPH_GRADH),
                    CF(SPH_BAL),  aux,          CF(SPH_AX),    CF(SPH_AY),   CF(SPH_AZ),  CF(SPH_ENGDOT),
                    CF(SPH_DT),   L.nbr,        L.cnt,         ctx->sup.map()};
        k_hydro64<<<sph_div_up(n, PT), PT, 0, ctx->stream>>>(n, a); ++ctx->launches;
    }
    SPH_CUDA(ctx, cudaGetLastError());
    return SPH_OK;
}

int sph_pass_gravity(sph_ctx *ctx, int build_lists) {
    if (build_lists) SPH_TRY(sph_build_grav_lists(ctx));
    GravLists &G = ctx->grav;
    Tree &t = ctx->tree;
    if (G.ng == 0) return SPH_OK;
    if (ctx->cfg.precision == SPH_PREC_MIXED) {
        // cell monopoles as double-float in the F2 scratch block (2 float4 per cell fit in 4 fields)
        if ((int64_t)t.n_cell_host * 2 > ctx->cap * 4) return sph_fail(ctx, SPH_ERR_CAPACITY, "cell pack scratch");
        float4 *ch = (float4 *)ctx->F2, *cl = ch + t.n_cell_host;
        const double gscale = 1.0;
        k_pack_cells32<<<2 * ctx->num_sms, 256, 0, ctx->stream>>>(t.meta, t.com, ctx->cfg.G, gscale, ch, cl); ++ctx->launches;
        k_grav32<<<G.ng, GT, 0, ctx->stream>>>(G.group_cell, t.start, t.count, ctx->xh, ctx->xl, CF(SPH_MASS),
                                               CF(SPH_SMTH), ch, cl, G.n_epj, G.off_epj, G.epj, G.n_spj, G.off_spj,
                                               G.spj, ctx->cfg.G, gscale, 1.0 / gscale, CF(SPH_GX), CF(SPH_GY),
                                               CF(SPH_GZ), CF(SPH_POT)); ++ctx->launches;
    } else {
        k_grav64<<<G.ng, GT, 0, ctx->stream>>>(G.group_cell, t.start, t.count, CF(SPH_X), CF(SPH_Y), CF(SPH_Z),
                                               CF(SPH_MASS), CF(SPH_SMTH), t.com, G.n_epj, G.off_epj, G.epj, G.n_spj,
                                               G.off_spj, G.spj, ctx->cfg.G, CF(SPH_GX), CF(SPH_GY), CF(SPH_GZ),
                                               CF(SPH_POT)); ++ctx->launches;
    }
    SPH_CUDA(ctx, cudaGetLastError());
    return SPH_OK;
}

// the step's dt of every run is in runs.dt_dev (set by sph_run_reduce_dt or the host)
int sph_kick_drift_predict(sph_ctx *ctx) {
    const int n = (int)ctx->n;
    k_kick_drift_predict<<<sph_div_up(n, 256), 256, 0, ctx->stream>>>(n, integ_args(ctx)); ++ctx->launches;
    SPH_CUDA(ctx, cudaGetLastError());
    return SPH_OK;
}

int sph_final_kick(sph_ctx *ctx) {
    const int n = (int)ctx->n;
    k_final_kick<<<sph_div_up(n, 256), 256, 0, ctx->stream>>>(n, integ_args(ctx), ctx->cfg.damping); ++ctx->launches;
    SPH_CUDA(ctx, cudaGetLastError());
    return SPH_OK;
}

// GI_universal::addExternalForce (GI.h:458-465) for the runs whose time is before ext_damp_tend
int sph_ext_force(sph_ctx *ctx) {
    if (!ctx->cfg.ext_damp) return SPH_OK;
    Runs &R = ctx->runs;
    std::vector<unsigned char> on(R.R);
    bool any = false;
    for (int r = 0; r < R.R; ++r) {
        on[r] = R.time[r] < ctx->cfg.ext_damp_tend;
        any = any || on[r];
    }
    if (!any) return SPH_OK;
    SPH_CUDA(ctx, cudaMemcpyAsync(R.damp, on.data(), R.R, cudaMemcpyHostToDevice, ctx->stream));
    const int n = (int)ctx->n;
    k_ext_force<<<sph_div_up(n, 256), 256, 0, ctx->stream>>>(n, integ_args(ctx), CF(SPH_DT), R.damp); ++ctx->launches;
    SPH_CUDA(ctx, cudaGetLastError());
    SPH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));   // `on` lives on the host stack
    return SPH_OK;
}

// getTimeStepGlobal (integral.h:4-20) for every run: min over the run's dt_i into runs.dt_dev and runs.dt
int sph_run_reduce_dt(sph_ctx *ctx) {
    Runs &R = ctx->runs;
    k_min_tiles<<<R.T, 256, 0, ctx->stream>>>(CF(SPH_DT), R.tiles, R.part); ++ctx->launches;
    k_min_runs<<<R.R, 256, 0, ctx->stream>>>(R.part, R.info, R.dt_dev); ++ctx->launches;
    std::vector<double> h(R.R);
    SPH_CUDA(ctx, cudaMemcpyAsync(h.data(), R.dt_dev, sizeof(double) * R.R, cudaMemcpyDeviceToHost, ctx->stream));
    SPH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    for (int r = 0; r < R.R; ++r) {
        const double d = h[r];
        if (!(d > 0.0) || !isfinite(d))
            return sph_fail(ctx, SPH_ERR_NONFINITE, "run %d: global dt is not a positive finite number (%g)", r, d);
        R.dt[r] = d;
    }
    return SPH_OK;
}

// conserved quantities per run: out[r * 8 + k] (k as sph_diagnostics)
int sph_run_diag(sph_ctx *ctx, double *out) {
    Runs &R = ctx->runs;
    k_diag_tiles<<<R.T, 256, 0, ctx->stream>>>(CF(SPH_X), CF(SPH_Y), CF(SPH_Z), CF(SPH_VX), CF(SPH_VY), CF(SPH_VZ),
                                               CF(SPH_MASS), CF(SPH_ENG), CF(SPH_POT), R.tiles, R.part);
    ++ctx->launches;
    k_diag_runs<<<sph_div_up(R.R * 8, 256), 256, 0, ctx->stream>>>(R.part, R.info, R.R, R.out); ++ctx->launches;
    SPH_CUDA(ctx, cudaMemcpyAsync(out, R.out, sizeof(double) * 8 * R.R, cudaMemcpyDeviceToHost, ctx->stream));
    SPH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return SPH_OK;
}

int sph_diag(sph_ctx *ctx, double out[8]) {
    std::vector<double> per(8 * (size_t)ctx->runs.R);
    SPH_TRY(sph_run_diag(ctx, per.data()));
    for (int k = 0; k < 8; ++k) {
        double v = 0.0;
        for (int r = 0; r < ctx->runs.R; ++r) v += per[(size_t)r * 8 + k];
        out[k] = v;
    }
    return SPH_OK;
}

// RealPtcl::initialize (class.h:196-199) for particles [off, off + n)
int sph_init_smth(sph_ctx *ctx, int64_t off, int64_t n) {
    k_init_smth<<<sph_div_up(n, 256), 256, 0, ctx->stream>>>((int)n, CF(SPH_MASS) + off, CF(SPH_DENS) + off,
                                                             CF(SPH_SMTH) + off, CF(SPH_GRADH) + off); ++ctx->launches;
    SPH_CUDA(ctx, cudaGetLastError());
    return SPH_OK;
}

// pair counts of the current lists: [0] gather-list pairs (one density or
// derivative pass), [1] symmetric-list pairs (hydro), [2] gravity i x (EPJ + SPJ)
// interactions, [3] cells, [4] gravity groups, [5] EPJ entries, [6] SPJ entries
int sph_work_counts(sph_ctx *ctx, int64_t out[8]) {
    for (int k = 0; k < 8; ++k) out[k] = 0;
    unsigned long long *d = (unsigned long long *)(ctx->scratch_d + 4096);
    SPH_CUDA(ctx, cudaMemsetAsync(d, 0, 6 * sizeof(unsigned long long), ctx->stream));
    const int n = (int)ctx->n;
    if (ctx->sup.valid) k_sum_cnt<<<2 * ctx->num_sms, 256, 0, ctx->stream>>>(n, ctx->sup.cnt, d + 3);
    if (ctx->lists[0].valid) k_sum_cnt<<<2 * ctx->num_sms, 256, 0, ctx->stream>>>(n, ctx->lists[0].cnt, d);
    if (ctx->lists[1].valid) k_sum_cnt<<<2 * ctx->num_sms, 256, 0, ctx->stream>>>(n, ctx->lists[1].cnt, d + 1);
    if (ctx->grav.counts_valid && ctx->grav.ng > 0) {
        k_sum_grav_pairs<<<2 * ctx->num_sms, 256, 0, ctx->stream>>>(ctx->grav.ng, ctx->grav.group_cell, ctx->tree.count,
                                                                    ctx->grav.n_epj, ctx->grav.n_spj, d + 2);
        k_sum_cnt<<<2 * ctx->num_sms, 256, 0, ctx->stream>>>(ctx->grav.ng, ctx->grav.n_epj, d + 4);
        k_sum_cnt<<<2 * ctx->num_sms, 256, 0, ctx->stream>>>(ctx->grav.ng, ctx->grav.n_spj, d + 5);
    }
    SPH_CUDA(ctx, cudaGetLastError());
    unsigned long long h[6];
    SPH_CUDA(ctx, cudaMemcpyAsync(h, d, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    SPH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    out[0] = (int64_t)h[0];
    out[1] = (int64_t)h[1];
    out[2] = (int64_t)h[2];
    out[3] = ctx->tree.n_cell_host;
    out[4] = ctx->grav.ng;
    out[5] = (int64_t)h[4];
    out[6] = (int64_t)h[5];
    out[7] = (int64_t)h[3];
    return SPH_OK;
}

// mixed-precision gravity with the walk fused into the force kernel
int sph_gravity_fused(sph_ctx *ctx) {
    SPH_TRY(sph_build_grav_groups(ctx));
    GravLists &G = ctx->grav;
    Tree &t = ctx->tree;
    if (G.ng == 0) return SPH_OK;
    if ((int64_t)t.n_cell_host * 2 > ctx->cap * 4) return sph_fail(ctx, SPH_ERR_CAPACITY, "cell pack scratch");
    float4 *chp = (float4 *)ctx->F2, *clp = chp + t.n_cell_host;
    k_pack_cells32<<<2 * ctx->num_sms, 256, 0, ctx->stream>>>(t.meta, t.com, ctx->cfg.G, 1.0, chp, clp);
    ++ctx->launches;
    // xh.w holds m * mscale: G m = xh.w * (G / mscale)
    const float gms = (float)(ctx->cfg.G / ctx->mscale);
    int *hs = (int *)ctx->host_scalars;
    // the 128-thread shape first; a walk whose front outgrew its ring (or a batch its buffers) flags
    // the error word, and the whole pass runs again with the 256-thread shape, which rewrites every
    // group's forces and counts
    for (int wide = 0; wide < 2; ++wide) {
        SPH_CUDA(ctx, cudaMemsetAsync(t.meta + META_ERR, 0, sizeof(int), ctx->stream));
        auto kern = wide ? k_grav_fused32<256> : k_grav_fused32<128>;
        kern<<<G.ng, wide ? 256 : 128, 0, ctx->stream>>>(G.group_cell, t.cinfo, t.com, t.rb, ctx->runs.prun, CF(SPH_X),
                                                         CF(SPH_Y), CF(SPH_Z), ctx->xh, ctx->xl, CF(SPH_SMTH), chp, clp,
                                                         gms, CF(SPH_GX), CF(SPH_GY), CF(SPH_GZ), CF(SPH_POT), G.n_epj,
                                                         G.n_spj, t.meta + META_ERR);
        ++ctx->launches;
        SPH_CUDA(ctx, cudaGetLastError());
        SPH_CUDA(ctx, cudaMemcpyAsync(hs, t.meta + META_ERR, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        SPH_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        if (!(hs[0] & ERR_GRAV_OVERFLOW)) break;
        if (wide) return sph_fail(ctx, SPH_ERR_CAPACITY, "gravity walk buffers overflowed");
    }
    G.counts_valid = true;
    return SPH_OK;
}

// ---------------------------------------------------------------------------
// Launch-shape autotuner for the mixed derivative and hydro kernels: threads per
// i-particle (1, 2 or 4) timed on the context's current state and lists, the
// fastest kept.  The fields the trial launches write are saved and restored.
extern "C" int sph_autotune(sph_ctx *ctx, int mode, int64_t params[8]) {
    if (!ctx || !params) return SPH_ERR_ARG;
    auto ok_tpi = [](int64_t v) { return v == 1 || v == 2 || v == 4; };
    if (mode == 1) {   // apply given choices
        if (!ok_tpi(params[0]) || !ok_tpi(params[1])) return sph_fail(ctx, SPH_ERR_ARG, "threads per particle must be 1, 2 or 4");
        ctx->tune.drvt_tpi = (int)params[0];
        ctx->tune.hydro_tpi = (int)params[1];
        return SPH_OK;
    }
    if (mode != 0) return sph_fail(ctx, SPH_ERR_ARG, "unknown autotune mode %d", mode);
    if (ctx->cfg.precision != SPH_PREC_MIXED) return sph_fail(ctx, SPH_ERR_STATE, "autotune tunes the mixed kernels");
    if (!ctx->uploaded || !ctx->have_forces || !ctx->lists[0].valid || !ctx->lists[1].valid || !ctx->xh)
        return sph_fail(ctx, SPH_ERR_STATE, "autotune needs the lists of a completed step (call it after sph_step)");
    cudaSetDevice(ctx->device);
    const int saved[] = {SPH_DIVV, SPH_ROTX, SPH_ROTY, SPH_ROTZ, SPH_GRADH, SPH_BAL,
                         SPH_AX,   SPH_AY,   SPH_AZ,   SPH_ENGDOT, SPH_DT};
    const int ns = (int)(sizeof(saved) / sizeof(saved[0]));
    const int64_t n = ctx->n;
    double *keep = nullptr;
    if (cudaMalloc((void **)&keep, sizeof(double) * n * ns) != cudaSuccess) {
        cudaGetLastError();
        return sph_fail(ctx, SPH_ERR_OOM, "autotune scratch");
    }
    for (int f = 0; f < ns; ++f)
        SPH_CUDA(ctx, cudaMemcpyAsync(keep + f * n, CF(saved[f]), sizeof(double) * n, cudaMemcpyDeviceToDevice,
                                      ctx->stream));
    const int choices[3] = {1, 2, 4};
    float best_ms[2] = {1e30f, 1e30f};
    int best[2] = {1, 1};
    int rc = SPH_OK;
    for (int which = 0; which < 2 && rc == SPH_OK; ++which) {
        for (int c = 0; c < 3 && rc == SPH_OK; ++c) {
            if (which == 0) ctx->tune.drvt_tpi = choices[c];
            else ctx->tune.hydro_tpi = choices[c];
            float ms = 0.0f;
            for (int rep = 0; rep < 4 && rc == SPH_OK; ++rep) {   // first launch warms up
                cudaEventRecord(ctx->ev_begin, ctx->stream);
                rc = which == 0 ? sph_pass_derivative(ctx, 0) : sph_pass_hydro(ctx, 0);
                cudaEventRecord(ctx->ev_end, ctx->stream);
                cudaEventSynchronize(ctx->ev_end);
                float e = 0.0f;
                cudaEventElapsedTime(&e, ctx->ev_begin, ctx->ev_end);
                if (rep > 0) ms += e / 3.0f;
            }
            params[2 + which * 3 + c] = (int64_t)(ms * 1000.0f);   // microseconds
            if (ms < best_ms[which]) {
                best_ms[which] = ms;
                best[which] = choices[c];
            }
        }
    }
    ctx->tune.drvt_tpi = best[0];
    ctx->tune.hydro_tpi = best[1];
    for (int f = 0; f < ns; ++f)
        cudaMemcpyAsync(CF(saved[f]), keep + f * n, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    cudaFree(keep);
    if (rc != SPH_OK) return rc;
    SPH_CUDA(ctx, cudaGetLastError());
    params[0] = best[0];
    params[1] = best[1];
    return SPH_OK;
}
