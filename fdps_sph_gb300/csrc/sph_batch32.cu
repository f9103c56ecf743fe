// Mixed-precision functor kernels for the batch entry points (sph_dispatch_* after
// sph_batch_set_precision(SPH_PREC_MIXED)).
//
// The same walks and results as the FP64 kernels of sph_batch.cu (the reference functors,
// force.h:9-23, 89-106, 113-147, 154-168), with the pair arithmetic of the device-resident mixed
// path: positions and velocities relative to the walk's first i-particle as double-floats (hi + lo
// FP32 pairs formed from the FP64 payload once per particle), pair terms in FP32 with the
// approximate root / reciprocal instructions, masses in units of one mass of the walk and the
// kernel normalisation of the i-particle factored out of the sums, FP32 partial sums of 32 terms
// added into compensated FP32 accumulators, and the per-particle epilogue (density floor and h, grad-h factor, dt, the normalisation) in FP64.  One
// block per walk, one thread per i-particle, the walk's j-list staged through shared memory.
#include "sph_batch.cuh"

using namespace sph;

namespace {

constexpr int WT = 128;

struct DF3 {   // a double-float 3-vector relative to the walk origin
    float hx, hy, hz, lx, ly, lz;
};

__device__ __forceinline__ DF3 rel3(const double *p, const double3 o) {
    DF3 r;
    float a, b;
    split_df(p[0] - o.x, a, b);
    r.hx = a;
    r.lx = b;
    split_df(p[1] - o.y, a, b);
    r.hy = a;
    r.ly = b;
    split_df(p[2] - o.z, a, b);
    r.hz = a;
    r.lz = b;
    return r;
}

__device__ __forceinline__ float dfd(float ah, float al, float bh, float bl) { return (ah - bh) + (al - bl); }

// CalcDensity: rho = max(5, norm sum m_j W), h = 1.2 (m / rho)^(1/3)
__global__ void __launch_bounds__(WT) k_walk_dens32(const int64_t *meta, const sph_epi_dens *epi,
                                                    JSrc<sph_epj_dens> epj, sph_result_dens *res) {
    __shared__ DF3 sp[WT];
    __shared__ float sm[WT];
    const int64_t *M = meta + 6 * blockIdx.x;
    const int64_t io = M[0], ni = M[1], jo = M[2], nj = M[3];
    if (ni <= 0) return;
    const double3 o = make_double3(epi[io].pos[0], epi[io].pos[1], epi[io].pos[2]);
    const double m0 = epi[io].mass > 0.0 ? epi[io].mass : 1.0;   // the walk's mass unit (FP32 range)
    for (int64_t i0 = 0; i0 < ni; i0 += WT) {
        const int64_t ii = i0 + threadIdx.x;
        const bool act = ii < ni;
        DF3 pi{};
        double hi = 1.0, mi = 1.0;
        if (act) {
            pi = rel3(epi[io + ii].pos, o);
            hi = epi[io + ii].smth;
            mi = epi[io + ii].mass;
        }
        const double Hd = SUPPORT * hi;
        const float invH = (float)(1.0 / Hd);
        float sh = 0.0f, sl = 0.0f, part = 0.0f;
        int cnt = 0;
        for (int64_t t0 = 0; t0 < nj; t0 += WT) {
            if (t0 + threadIdx.x < nj) {
                const sph_epj_dens &q = epj[jo + t0 + threadIdx.x];
                sp[threadIdx.x] = rel3(q.pos, o);
                sm[threadIdx.x] = (float)(q.mass / m0);
            }
            __syncthreads();
            const int tn = (int)min((int64_t)WT, nj - t0);
            for (int t = 0; t < tn; ++t) {
                const DF3 q = sp[t];
                const float dx = dfd(q.hx, q.lx, pi.hx, pi.lx), dy = dfd(q.hy, q.ly, pi.hy, pi.ly),
                            dz = dfd(q.hz, q.lz, pi.hz, pi.lz);
                const float s = sqrt_a(dx * dx + dy * dy + dz * dz) * invH;
                const float p = fmaxf(1.0f - s, 0.0f), p2 = p * p, p4 = p2 * p2;
                part = fmaf(sm[t], (1.0f + s * (8.0f + s * (25.0f + s * 32.0f))) * (p4 * p4), part);
                if (++cnt == 32) {
                    df_add(sh, sl, part);
                    part = 0.0f;
                    cnt = 0;
                }
            }
            __syncthreads();
        }
        df_add(sh, sl, part);
        if (act) {
            const double d = fmax(DENS_FLOOR, ((double)sh + (double)sl) * m0 * kernel_norm(Hd));
            res[io + ii].dens = d;
            res[io + ii].smth = SMTH_COEF * cbrt(mi / d);
        }
    }
}

// CalcDerivative + grad-h factor: div v, rot v, grad_smth (force.h:89-106)
__global__ void __launch_bounds__(WT) k_walk_drvt32(const int64_t *meta, const sph_epi_drvt *epi,
                                                    JSrc<sph_epj_drvt> epj, sph_result_drvt *res) {
    __shared__ DF3 sp[WT], sv[WT];
    __shared__ float sm[WT];
    const int64_t *M = meta + 6 * blockIdx.x;
    const int64_t io = M[0], ni = M[1], jo = M[2], nj = M[3];
    if (ni <= 0) return;
    const double3 o = make_double3(epi[io].pos[0], epi[io].pos[1], epi[io].pos[2]);
    const double3 ov = make_double3(epi[io].vel[0], epi[io].vel[1], epi[io].vel[2]);
    const double m0 = (nj > 0 && epj[jo].mass > 0.0) ? epj[jo].mass : 1.0;   // the walk's mass unit
    for (int64_t i0 = 0; i0 < ni; i0 += WT) {
        const int64_t ii = i0 + threadIdx.x;
        const bool act = ii < ni;
        DF3 pi{}, vi{};
        double hi = 1.0, rhoi = 1.0;
        if (act) {
            pi = rel3(epi[io + ii].pos, o);
            vi = rel3(epi[io + ii].vel, ov);
            hi = epi[io + ii].smth;
            rhoi = epi[io + ii].dens;
        }
        const double Hd = SUPPORT * hi;
        const float Hf = (float)Hd, invH = (float)(1.0 / Hd), ceps = (float)(1.0e-6 * hi);
        float Dh[5] = {0, 0, 0, 0, 0}, Dl[5] = {0, 0, 0, 0, 0}, P[5] = {0, 0, 0, 0, 0};
        int cnt = 0;
        for (int64_t t0 = 0; t0 < nj; t0 += WT) {
            if (t0 + threadIdx.x < nj) {
                const sph_epj_drvt &q = epj[jo + t0 + threadIdx.x];
                sp[threadIdx.x] = rel3(q.pos, o);
                sv[threadIdx.x] = rel3(q.vel, ov);
                sm[threadIdx.x] = (float)(q.mass / m0);
            }
            __syncthreads();
            const int tn = (int)min((int64_t)WT, nj - t0);
            for (int t = 0; t < tn; ++t) {
                const DF3 q = sp[t], u = sv[t];
                const float dx = dfd(pi.hx, pi.lx, q.hx, q.lx), dy = dfd(pi.hy, pi.ly, q.hy, q.ly),
                            dz = dfd(pi.hz, pi.lz, q.hz, q.lz);
                const float wx = dfd(u.hx, u.lx, vi.hx, vi.lx), wy = dfd(u.hy, u.ly, vi.hy, vi.ly),
                            wz = dfd(u.hz, u.lz, vi.hz, vi.lz);   // v_j - v_i
                const float rr2 = dx * dx + dy * dy + dz * dz;
                const float r = sqrt_a(rr2);
                float w, g;
                wendland_poly_f(r * invH, w, g);
                const float gf = g * rcp_a(r * Hf + ceps);
                const float m = sm[t];
                P[0] = fmaf(m * gf, wx * dx + wy * dy + wz * dz, P[0]);
                P[1] = fmaf(m * gf, wy * dz - wz * dy, P[1]);
                P[2] = fmaf(m * gf, wz * dx - wx * dz, P[2]);
                P[3] = fmaf(m * gf, wx * dy - wy * dx, P[3]);
                P[4] = fmaf(m, 3.0f * w + gf * rr2, P[4]);
                if (++cnt == 32) {
#pragma unroll
                    for (int k = 0; k < 5; ++k) {
                        df_add(Dh[k], Dl[k], P[k]);
                        P[k] = 0.0f;
                    }
                    cnt = 0;
                }
            }
            __syncthreads();
        }
        if (act) {
            double D[5];
            const double norm = m0 * kernel_norm(Hd);
#pragma unroll
            for (int k = 0; k < 5; ++k) {
                df_add(Dh[k], Dl[k], P[k]);
                D[k] = ((double)Dh[k] + (double)Dl[k]) * norm;
            }
            const double gs = -D[4] / hi;
            sph_result_drvt &out = res[io + ii];
            out.grad_smth = 1.0 / (1.0 + hi * gs / (3.0 * rhoi));
            out.div_v = D[0] / rhoi;
            out.rot_v[0] = D[1] / rhoi;
            out.rot_v[1] = D[2] / rhoi;
            out.rot_v[2] = D[3] / rhoi;
        }
    }
}

// CalcHydroForce: acceleration, du/dt, dt (force.h:113-147)
struct HJ {
    DF3 p, v;
    float m, H, invH, rho, A, cs, f, bal;
};

__global__ void __launch_bounds__(WT) k_walk_hydro32(const int64_t *meta, const sph_epi_hydro *epi,
                                                     JSrc<sph_epj_hydro> epj, sph_result_hydro *res) {
    __shared__ HJ sj[WT];
    const int64_t *M = meta + 6 * blockIdx.x;
    const int64_t io = M[0], ni = M[1], jo = M[2], nj = M[3];
    if (ni <= 0) return;
    const double3 o = make_double3(epi[io].pos[0], epi[io].pos[1], epi[io].pos[2]);
    const double3 ov = make_double3(epi[io].vel[0], epi[io].vel[1], epi[io].vel[2]);
    const double m0 = (nj > 0 && epj[jo].mass > 0.0) ? epj[jo].mass : 1.0;   // the walk's mass unit
    for (int64_t i0 = 0; i0 < ni; i0 += WT) {
        const int64_t ii = i0 + threadIdx.x;
        const bool act = ii < ni;
        DF3 pi{}, vi{};
        double hi = 1.0, rhoi = 1.0, Pi = 0.0, ci = 0.0, fi = 1.0, bi = 0.0;
        if (act) {
            const sph_epi_hydro &I = epi[io + ii];
            pi = rel3(I.pos, o);
            vi = rel3(I.vel, ov);
            hi = I.smth;
            rhoi = I.dens;
            Pi = I.pres;
            ci = I.snds;
            fi = I.grad_smth;
            bi = I.Bal;
        }
        const double Hd = SUPPORT * hi;
        const float Hi = (float)Hd, invHi = (float)(1.0 / Hd), cepsi = (float)(1.0e-6 * hi);
        const float Ai = (float)(fi * Pi / (rhoi * rhoi)), rhof = (float)rhoi, cf = (float)ci, ff = (float)fi,
                    bf = (float)bi;
        float Dh[4] = {0, 0, 0, 0}, Dl[4] = {0, 0, 0, 0}, P[4] = {0, 0, 0, 0};
        float vmax = 0.0f;
        int cnt = 0;
        for (int64_t t0 = 0; t0 < nj; t0 += WT) {
            if (t0 + threadIdx.x < nj) {
                const sph_epj_hydro &q = epj[jo + t0 + threadIdx.x];
                HJ h;
                h.p = rel3(q.pos, o);
                h.v = rel3(q.vel, ov);
                const double Hj = SUPPORT * q.smth;
                h.m = (float)(q.mass / m0);
                h.H = (float)Hj;
                h.invH = (float)(1.0 / Hj);
                h.rho = (float)q.dens;
                h.A = (float)(q.grad_smth * q.pres / (q.dens * q.dens));
                h.cs = (float)q.snds;
                h.f = (float)q.grad_smth;
                h.bal = (float)q.Bal;
                sj[threadIdx.x] = h;
            }
            __syncthreads();
            const int tn = (int)min((int64_t)WT, nj - t0);
            for (int t = 0; t < tn; ++t) {
                const HJ &J = sj[t];
                const float dx = dfd(pi.hx, pi.lx, J.p.hx, J.p.lx), dy = dfd(pi.hy, pi.ly, J.p.hy, J.p.ly),
                            dz = dfd(pi.hz, pi.lz, J.p.hz, J.p.lz);
                const float wx = dfd(vi.hx, vi.lx, J.v.hx, J.v.lx), wy = dfd(vi.hy, vi.ly, J.v.hy, J.v.ly),
                            wz = dfd(vi.hz, vi.lz, J.v.hz, J.v.lz);
                const float rr2 = dx * dx + dy * dy + dz * dz;
                const float r = sqrt_a(rr2);
                const float dvdr = wx * dx + wy * dy + wz * dz;
                const float w = (dvdr < 0.0f) ? dvdr * rcp_a(r) : 0.0f;
                const float vsig = cf + J.cs - 3.0f * w;
                vmax = fmaxf(vmax, vsig);
                const float AV = -0.5f * vsig * w * rcp_a(0.5f * (rhof + J.rho)) * 0.5f * (bf + J.bal);
                float wi_, gi_, wj_, gj_;
                wendland_poly_f(r * invHi, wi_, gi_);
                wendland_poly_f(r * J.invH, wj_, gj_);
                const float nr = Hi * J.invH;   // the j kernel's normalisation relative to the i kernel's
                const float gfi = gi_ * rcp_a(r * Hi + cepsi);
                const float gfj = (nr * nr * nr) * gj_ * rcp_a(r * J.H + 4.0e-7f * J.H);
                const float gws = 0.5f * (gfi * ff + gfj * J.f);
                const float coef = J.m * (Ai * gfi + J.A * gfj + AV * gws);
                P[0] = fmaf(-coef, dx, P[0]);
                P[1] = fmaf(-coef, dy, P[1]);
                P[2] = fmaf(-coef, dz, P[2]);
                P[3] = fmaf(J.m * (Ai + 0.5f * AV) * gws, dvdr, P[3]);
                if (++cnt == 32) {
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        df_add(Dh[k], Dl[k], P[k]);
                        P[k] = 0.0f;
                    }
                    cnt = 0;
                }
            }
            __syncthreads();
        }
        if (act) {
            const double norm = m0 * kernel_norm(Hd);
            double D[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                df_add(Dh[k], Dl[k], P[k]);
                D[k] = ((double)Dh[k] + (double)Dl[k]) * norm;
            }
            sph_result_hydro &out = res[io + ii];
            out.acc[0] = D[0];
            out.acc[1] = D[1];
            out.acc[2] = D[2];
            out.eng_dot = D[3];
            out.dt = C_CFL * 2.0 * hi / (double)vmax;
        }
    }
}

// CalcGravityForce<EPJ::Grav> then <SPJMonopole> (force.h:154-168): G m folded into the tile
__global__ void __launch_bounds__(WT) k_walk_grav32(const int64_t *meta, const sph_epi_grav *epi,
                                                    JSrc<sph_epj_grav> epj, JSrc<sph_spj_monopole> spj,
                                                    sph_result_grav *res) {
    __shared__ DF3 sp[WT];
    __shared__ float sg[WT];
    const double G = 6.67e-11;   // force.h:171-172
    const int64_t *M = meta + 6 * blockIdx.x;
    const int64_t io = M[0], ni = M[1], jo = M[2], nj = M[3], so = M[4], ns = M[5];
    if (ni <= 0) return;
    const double3 o = make_double3(epi[io].pos[0], epi[io].pos[1], epi[io].pos[2]);
    // G m in units of the walk's first EPJ mass (or SPJ mass) keeps the FP32 products in range
    const double gscale = nj > 0 ? G * epj[jo].mass : (ns > 0 ? G * spj[so].mass : G);
    for (int64_t i0 = 0; i0 < ni; i0 += WT) {
        const int64_t ii = i0 + threadIdx.x;
        const bool act = ii < ni;
        DF3 pi{};
        float e2 = 1.0f;
        if (act) {
            pi = rel3(epi[io + ii].pos, o);
            e2 = (float)epi[io + ii].eps2;
        }
        float Dh[4] = {0, 0, 0, 0}, Dl[4] = {0, 0, 0, 0}, P[4] = {0, 0, 0, 0};
        int cnt = 0;
        for (int pass = 0; pass < 2; ++pass) {
            const int64_t nl = pass == 0 ? nj : ns;
            for (int64_t t0 = 0; t0 < nl; t0 += WT) {
                if (t0 + threadIdx.x < nl) {
                    const double *pp = pass == 0 ? epj[jo + t0 + threadIdx.x].pos : spj[so + t0 + threadIdx.x].pos;
                    const double mm = pass == 0 ? epj[jo + t0 + threadIdx.x].mass : spj[so + t0 + threadIdx.x].mass;
                    sp[threadIdx.x] = rel3(pp, o);
                    sg[threadIdx.x] = (float)(G * mm / gscale);
                }
                __syncthreads();
                const int tn = (int)min((int64_t)WT, nl - t0);
                for (int t = 0; t < tn; ++t) {
                    const DF3 q = sp[t];
                    const float dx = dfd(pi.hx, pi.lx, q.hx, q.lx), dy = dfd(pi.hy, pi.ly, q.hy, q.ly),
                                dz = dfd(pi.hz, pi.lz, q.hz, q.lz);
                    const float ri = rsqrt_a(fmaf(dx, dx, fmaf(dy, dy, fmaf(dz, dz, e2))));
                    const float mri = sg[t] * ri;
                    const float mr3 = mri * ri * ri;
                    P[0] = fmaf(-mr3, dx, P[0]);
                    P[1] = fmaf(-mr3, dy, P[1]);
                    P[2] = fmaf(-mr3, dz, P[2]);
                    P[3] -= mri;
                    if (++cnt == 32) {
#pragma unroll
                        for (int k = 0; k < 4; ++k) {
                            df_add(Dh[k], Dl[k], P[k]);
                            P[k] = 0.0f;
                        }
                        cnt = 0;
                    }
                }
                __syncthreads();
            }
        }
        if (act) {
            sph_result_grav &out = res[io + ii];
            double D[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                df_add(Dh[k], Dl[k], P[k]);
                D[k] = ((double)Dh[k] + (double)Dl[k]) * gscale;
            }
            out.acc[0] = D[0];
            out.acc[1] = D[1];
            out.acc[2] = D[2];
            out.pot = D[3];
            out.dt = 1.0e30;   // RESULT::Grav::clear(), dt untouched by the functor
        }
    }
}

}  // namespace

namespace sph {

// launchers for sph_batch.cu: one block per walk on the tag's stream
void batch32_dens(int n_walk, cudaStream_t st, const int64_t *meta, const sph_epi_dens *epi, JSrc<sph_epj_dens> epj,
                  sph_result_dens *res) {
    k_walk_dens32<<<n_walk, WT, 0, st>>>(meta, epi, epj, res);
}
void batch32_drvt(int n_walk, cudaStream_t st, const int64_t *meta, const sph_epi_drvt *epi, JSrc<sph_epj_drvt> epj,
                  sph_result_drvt *res) {
    k_walk_drvt32<<<n_walk, WT, 0, st>>>(meta, epi, epj, res);
}
void batch32_hydro(int n_walk, cudaStream_t st, const int64_t *meta, const sph_epi_hydro *epi,
                   JSrc<sph_epj_hydro> epj, sph_result_hydro *res) {
    k_walk_hydro32<<<n_walk, WT, 0, st>>>(meta, epi, epj, res);
}
void batch32_grav(int n_walk, cudaStream_t st, const int64_t *meta, const sph_epi_grav *epi, JSrc<sph_epj_grav> epj,
                  JSrc<sph_spj_monopole> spj, sph_result_grav *res) {
    k_walk_grav32<<<n_walk, WT, 0, st>>>(meta, epi, epj, spj, res);
}

}  // namespace sph
