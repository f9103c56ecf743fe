/* CPU oracle for the FDPS_SPH per-step interaction path -- TEST INFRASTRUCTURE.
 *
 * Plain-C restatement of the reference's algorithm; each function cites the
 * reference file:line it follows.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg may load this library, and only as the checker
 * or baseline.  Compiled with -ffp-contract=off so that every floating-point
 * operation is one IEEE-754 rounding: the tree/key/list decisions below are a
 * bit-exact specification that the device code reproduces with explicit
 * round-to-nearest intrinsics.
 */
#include "sph_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define F(s, f) ((s)->F + (int64_t)(f) * (s)->n)

static const double OR_SUPPORT = 2.5;            /* kernel.h:36-38 */
static const double OR_SMTH_COEF = 1.2;              /* param.h:9 */
static const double OR_CFL = 0.3;                /* param.h:10 */
static const double OR_AV_STRENGTH = 1.0;        /* param.h:17 */
static const double OR_DENS_FLOOR = 5.0;         /* force.h:18-20 (FLAG_GI) */
static const int OR_KEY_LEVELS = 21;             /* 3 x 21-bit Morton key */

int or_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* math helpers: mathfunc.h:4-57                                              */
static inline double or_plus(double a) { return (a > 0) ? a : 0; }
static inline double or_pow7(double a) { const double a3 = a * a * a; return a3 * a3 * a; }
static inline double or_pow8(double a) { const double a2 = a * a; const double a4 = a2 * a2; return a4 * a4; }
static inline double or_pi(void) { return atan(1.0) * 4.0; }                 /* mathfunc.h:4 */
static inline double or_max(double a, double b) { return (a < b) ? b : a; }  /* std::max */
static inline double or_min(double a, double b) { return (b < a) ? b : a; }  /* std::min */
static inline double or_dot(double ax, double ay, double az, double bx, double by, double bz) {
    return ax * bx + ay * by + az * bz;   /* PS::F64vec operator* : (x*x + y*y) + z*z */
}

/* Wendland C6 kernel, kernel.h:8-19 */
double or_kernel_W(double dx, double dy, double dz, double h) {
    const double H = OR_SUPPORT * h;
    const double s = sqrt(or_dot(dx, dy, dz, dx, dy, dz)) / H;
    double r = (1.0 + s * (8.0 + s * (25.0 + s * (32.0)))) * or_pow8(or_plus(1.0 - s));
    r *= (1365. / 64.) / (H * H * H * or_pi());
    return r;
}

/* Wendland C6 gradient, kernel.h:22-34 */
void or_kernel_gradW(double dx, double dy, double dz, double h, double g[3]) {
    const double H = OR_SUPPORT * h;
    const double rr = sqrt(or_dot(dx, dy, dz, dx, dy, dz));
    const double s = rr / H;
    double r = or_pow7(or_plus(1.0 - s)) * (or_plus(1.0 - s) * (8.0 + s * (50.0 + s * (96.0))) -
                                            8.0 * (1.0 + s * (8.0 + s * (25.0 + s * (32.0)))));
    r *= (1365. / 64.) / (H * H * H * or_pi());
    const double den = rr * H + 1.0e-6 * h;
    g[0] = dx * r / den;
    g[1] = dy * r / den;
    g[2] = dz * r / den;
}

/* ------------------------------------------------------------------------ */
/* EoS                                                                        */

/* std::lower_bound: first index k with !(ax[k] < v), interpolation.h:39-46 */
static int or_lower_bound(const double *ax, int n, double v) {
    int lo = 0, len = n;
    while (len > 0) {
        const int half = len >> 1;
        if (ax[lo + half] < v) {
            lo += half + 1;
            len -= half + 1;
        } else {
            len = half;
        }
    }
    return lo;
}

/* BilinearInterpolation::interpolate, interpolation.h:33-102.  The interior
 * test excludes index 0 and the last index, so the first and last intervals
 * of each axis (and anything outside the table) return the corner value. */
double or_table_lookup(const double *rho_ax, int n_rho, const double *u_ax, int n_u, const double *plane,
                       double rho, double u) {
    int li = or_lower_bound(rho_ax, n_rho, rho);
    int ci = or_lower_bound(u_ax, n_u, u);
    if (li > n_rho - 1) li = n_rho - 1;   /* interpolation.h:48-54 */
    if (ci > n_u - 1) ci = n_u - 1;
    if (li < n_rho - 1 && ci < n_u - 1 && li > 0 && ci > 0) {
        const double xi = (rho - rho_ax[li - 1]) / (rho_ax[li] - rho_ax[li - 1]);
        const double eta = (u - u_ax[ci - 1]) / (u_ax[ci] - u_ax[ci - 1]);
        return (1 - xi) * (1 - eta) * plane[(int64_t)(li - 1) * n_u + (ci - 1)] +
               xi * (1 - eta) * plane[(int64_t)li * n_u + (ci - 1)] +
               (1 - xi) * eta * plane[(int64_t)(li - 1) * n_u + ci] +
               xi * eta * plane[(int64_t)li * n_u + ci];
    }
    return plane[(int64_t)li * n_u + ci];
}

/* Analytic Tillotson.  The two branches are the reference's P_co and P_ex
 * (EoS.h:91-103) in their operation order, pinned to the reference's own
 * arithmetic by tests/golden/tillotson.npz.  The reference never selects
 * between them (they are dead code there), so the regime rule is this
 * project's, taken from the published equation the reference cites
 * (Brundage 2013, EoS.h:226-227; Tillotson 1962): compressed (rho >= rho0) or
 * cold-expanded (u <= uiv) states use P_co, hot-expanded states (u >= ucv)
 * use P_ex, and the region uiv < u < ucv for rho < rho0 blends the two
 * linearly in u.  The sound speed is also this project's definition:
 * c^2 = dP/drho|_u + P/rho^2 dP/du|_rho of the same expressions, floored at
 * 1e-2 A/rho0.  The reference's Tillotson class itself reads a table
 * (EoS.h:241-247); this analytic mode is used when a run asks for the
 * Tillotson parameters rather than a table. */
static void or_tillotson(const double *p, double rho, double u, double *P, double *cs) {
    const double rho0 = p[0], u0 = p[1], uiv = p[2], ucv = p[3], A = p[4], B = p[5], a = p[6], b = p[7],
                 alpha = p[8], beta = p[9];
    const double eta = rho / rho0;
    const double mu = eta - 1.0;
    const double om = u / u0 / eta / eta + 1.0;   /* operation order of P_co / P_ex, EoS.h:91-103 */
    /* compressed branch */
    const double Pc = (a + b / om) * rho * u + A * mu + B * mu * mu;
    const double dPc_drho = (a + b / om) * u + 2.0 * b * u * (om - 1.0) / (om * om) + (A + 2.0 * B * mu) / rho0;
    const double dPc_du = (a + b / om) * rho - rho * b * (om - 1.0) / (om * om);
    double Pv, dPdrho, dPdu;
    if (rho >= rho0 || u <= uiv) {
        Pv = Pc; dPdrho = dPc_drho; dPdu = dPc_du;
    } else {
        const double z = 1.0 / eta - 1.0;
        const double E1 = exp(-alpha * z);
        const double E2 = exp(-beta * z * z);
        const double Q = b * rho * u / om + A * mu * E1;
        const double Pe = a * rho * u + Q * E2;
        const double dQ = b * u / om + 2.0 * b * u * (om - 1.0) / (om * om) + A / rho0 * E1 +
                          A * mu * alpha * E1 * (z + 1.0) / rho;
        const double dPe_drho = a * u + dQ * E2 + Q * 2.0 * beta * z * (z + 1.0) * E2 / rho;
        const double dPe_du = a * rho + E2 * (b * rho / om - b * rho * (om - 1.0) / (om * om));
        if (u >= ucv) {
            Pv = Pe; dPdrho = dPe_drho; dPdu = dPe_du;
        } else {
            const double w = ucv - uiv;
            Pv = ((u - uiv) * Pe + (ucv - u) * Pc) / w;
            dPdrho = ((u - uiv) * dPe_drho + (ucv - u) * dPc_drho) / w;
            dPdu = (Pe - Pc + (u - uiv) * dPe_du + (ucv - u) * dPc_du) / w;
        }
    }
    double c2 = dPdrho + Pv / (rho * rho) * dPdu;
    const double c2min = 1.0e-2 * A / rho0;
    if (!(c2 > c2min)) c2 = c2min;
    *P = Pv;
    *cs = sqrt(c2);
}

/* CalcPressure per particle, force.h:26-32 -> EoS_t::Pressure/SoundSpeed */
void or_eos_eval(const or_material *m, double rho, double u, double *P, double *cs) {
    if (m->kind == 0) {
        /* ANEOS / Tillotson table classes: EoS.h:241-247, 394-400 (columns 3 and 4) */
        *P = or_table_lookup(m->rho, m->n_rho, m->u, m->n_u, m->pres, rho, u);
        *cs = or_table_lookup(m->rho, m->n_rho, m->u, m->n_u, m->snds, rho, u);
    } else if (m->kind == 1) {
        or_tillotson(m->par, rho, u, P, cs);
    } else {
        /* IdealGas, EoS.h:37-49 */
        const double g = m->par[0];
        *P = (g - 1.0) * rho * u;
        *cs = sqrt(g * (g - 1.0) * u);
    }
}

/* ------------------------------------------------------------------------ */
/* Mode-2 EoS surface: Temperature, Entropy, InternalEnergy                  */

/* EoS_t::Temperature / Entropy of the table classes: bilinear on columns 2 and
 * 5 (EoS.h:254-260, 407-413); IdealGas returns 0 (EoS.h:55-61). */
double or_eos_temperature(const or_material *m, double rho, double u) {
    if (m->kind == 2) return 0.0;
    if (m->kind != 0 || !m->temp) return NAN;
    return or_table_lookup(m->rho, m->n_rho, m->u, m->n_u, m->temp, rho, u);
}

double or_eos_entropy(const or_material *m, double rho, double u) {
    if (m->kind == 2) return 0.0;
    if (m->kind != 0 || !m->ent) return NAN;
    return or_table_lookup(m->rho, m->n_rho, m->u, m->n_u, m->ent, rho, u);
}

/* get_neighbors_restricted_indices(v, value, grid_length, bound)
 * (interpolation.h:131-182), literally: a forward scan for the first line with
 * v >= value ("upper"), a scan from the end for the last line with v <= value
 * ("lower"), in the reference's unsigned 32-bit index arithmetic. */
static void or_restricted_bounds(const double *v, int64_t size, double value, uint32_t G, int upper, uint32_t *b1,
                                 uint32_t *b2) {
    uint32_t lo = 0, hi = 0;
    if (upper) {
        for (int64_t a = 0; a < size; ++a)
            if (v[a] >= value) {
                lo = (uint32_t)a;
                hi = (uint32_t)a + G;
                if ((uint64_t)hi > (uint64_t)(size - 1)) hi = (uint32_t)(size - 1);
                break;
            }
    } else {
        for (int64_t a = 0; a < size; ++a)
            if (v[size - 1 - a] <= value) {
                lo = (uint32_t)(size - 1) - (uint32_t)a - (G - 1u);
                hi = lo + G;
                if (hi == 0) hi = G;
                break;
            }
    }
    if (lo == 0 && hi == 0) {
        lo = 0;
        hi = G;
    }
    *b1 = lo;
    *b2 = hi;
}

/* slice(v, m, n) (interpolation.h:17-25) reads [m, n]: defined for 0 <= m <= n + 1 <= size */
static int or_slice_ok(uint32_t b1, uint32_t b2, int64_t size) {
    const int64_t m = (int32_t)b1, n = (int32_t)b2;
    return m >= 0 && m <= n + 1 && n + 1 <= size;
}

/* abs() of a double as the reference's translation unit resolves it (int
 * abs(int) of the truncated value): defined for -2^31 < d < 2^31 */
static int or_int_abs(double d, int64_t *out) {
    if (!(d > -2147483648.0 && d < 2147483648.0)) return 0;
    const int64_t t = (int64_t)d;
    *out = t < 0 ? -t : t;
    return 1;
}

/* get_var2_neighbors (interpolation.h:186-238): positions (p0, p1) in the slice
 * around its entry nearest to `given` (first nearest in scan order).  Returns
 * 0 where the reference's distance arithmetic is undefined. */
static int or_var2_pair(const double *sl, int64_t L, double given, uint32_t G, int abs_mode, int32_t *p0, int32_t *p1) {
    double min_d = 0.0;
    uint32_t idx = 0;
    int ok = 1;
    for (int64_t a = 0; a < L; ++a) {
        const double d = given - sl[a];
        if (a == 0) {
            min_d = d;
            idx = 0;
            continue;
        }
        int closer;
        if (abs_mode == 0) {
            int64_t di = 0, dm = 0;
            ok &= or_int_abs(d, &di);
            ok &= or_int_abs(min_d, &dm);
            closer = di < dm;
        } else {
            closer = fabs(d) < fabs(min_d);
        }
        if (closer) {
            min_d = d;
            idx = (uint32_t)a;
        }
    }
    uint32_t f, s;
    if (min_d < 0) {
        if (idx <= 0) { f = idx; s = idx + 1; }
        else if (idx + 1 == G) { f = idx - 2; s = idx - 1; }
        else { f = idx - 1; s = idx; }
    } else if (min_d > 0) {
        if (idx + 1 == G) { f = idx - 2; s = idx - 1; }
        else { f = idx; s = idx + 1; }
    } else {
        if (idx >= G - 1) { f = idx - 2; s = idx - 1; }
        else { f = idx - 1; s = idx + 1; }
    }
    *p0 = (int32_t)f;
    *p1 = (int32_t)s;
    return ok;
}

/* linear_interpolate (interpolation.h:254-262) */
static double or_lerp(double x1, double x2, double x, double q1, double q2) {
    return (((x2 - x) / (x2 - x1)) * q1) + (((x - x1) / (x2 - x1)) * q2);
}

/* RestrictedBilinearInterpolation::interpolate (interpolation.h:265-334) with
 * var1 = line densities, var2 = line entropies, var3 = line energies, as
 * InternalEnergy calls it (EoS.h:249-252, 402-405); IdealGas returns 0
 * (EoS.h:51-53).  The analytic Tillotson mode has no entropy data: NaN. */
double or_eos_internal_energy(const or_material *m, double rho, double s, int grid, int abs_mode, int *undef) {
    *undef = 0;
    if (m->kind == 2) return 0.0;
    if (m->kind != 0 || !m->ent || !m->line_rho || !m->line_u || grid < 1) {
        *undef = 1;
        return NAN;
    }
    const int64_t size = (int64_t)m->n_rho * m->n_u;
    const double *vr = m->line_rho, *ve = m->ent, *vu = m->line_u;
    const uint32_t G = (uint32_t)grid;
    uint32_t l1, l2, h1, h2;
    or_restricted_bounds(vr, size, rho, G, 0, &l1, &l2);
    or_restricted_bounds(vr, size, rho, G, 1, &h1, &h2);
    if (!or_slice_ok(l1, l2, size) || !or_slice_ok(h1, h2, size)) {
        *undef = 1;
        return NAN;
    }
    const int64_t Ll = (int64_t)(int32_t)l2 - (int32_t)l1 + 1, Lh = (int64_t)(int32_t)h2 - (int32_t)h1 + 1;
    int32_t a0, a1, c0, c1;
    const int ok = or_var2_pair(ve + l1, Ll, s, G, abs_mode, &a0, &a1) &
                   or_var2_pair(ve + h1, Lh, s, G, abs_mode, &c0, &c1);
    if (!ok || Ll < 1 || Lh < 1 || a0 < 0 || a1 < 0 || c0 < 0 || c1 < 0 || a0 >= Ll || a1 >= Ll || c0 >= Lh ||
        c1 >= Lh) {
        *undef = 1;
        return NAN;
    }
    const double e1 = or_lerp(ve[l1 + a0], ve[l1 + a1], s, vu[l1 + a0], vu[l1 + a1]);
    const double e2 = or_lerp(ve[h1 + c0], ve[h1 + c1], s, vu[h1 + c0], vu[h1 + c1]);
    return or_lerp(vr[l1], vr[h1], rho, e1, e2);
}

/* SetConstantEntropy (force.h:55-65: tag 0 -> mantle, else core; the material
 * slot is the tag) and CalcAll (force.h:73-84) */
int64_t or_entropy_step(or_system *s, const or_config *cfg) {
    const int64_t n = s->n;
    const double *dens = F(s, OR_DENS);
    double *eng = F(s, OR_ENG), *ent = F(s, OR_ENT), *temp = F(s, OR_TEMP);
    int64_t bad = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : bad)
    for (int64_t i = 0; i < n; ++i) {
        const or_material *m = &cfg->mat[s->mat[i]];
        const double e = s->mat[i] == 0 ? cfg->mantle_entropy : cfg->core_entropy;
        int undef;
        const double u = or_eos_internal_energy(m, dens[i], e, cfg->entropy_grid, cfg->entropy_abs, &undef);
        ent[i] = e;
        eng[i] = u;
        temp[i] = or_eos_temperature(m, dens[i], u);
        bad += (undef || !isfinite(u)) ? 1 : 0;
    }
    return bad;
}

/* ------------------------------------------------------------------------ */
/* Morton keys and sort (FDPS tree construction; project specification)      */

void or_root_box(const double *x, const double *y, const double *z, int64_t n, or_rootbox *rb) {
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    const double *p[3] = {x, y, z};
    for (int d = 0; d < 3; ++d)
        for (int64_t i = 0; i < n; ++i) {
            const double v = p[d][i];
            if (v < lo[d]) lo[d] = v;
            if (v > hi[d]) hi[d] = v;
        }
    double L = 0.0;
    for (int d = 0; d < 3; ++d) {
        const double e = hi[d] - lo[d];
        if (e > L) L = e;
    }
    if (!(L > 0.0)) L = 1.0;
    const double half = L * 0.50048828125;   /* 0.5 * (1 + 2^-10) */
    for (int d = 0; d < 3; ++d) rb->root_lo[d] = (lo[d] + hi[d]) * 0.5 - half;
    rb->root_len = half + half;
    rb->scale = 2097152.0 / rb->root_len;
}

static inline uint64_t or_spread3(uint64_t v) {
    v &= 0x1fffffULL;
    v = (v | (v << 32)) & 0x1f00000000ffffULL;
    v = (v | (v << 16)) & 0x1f0000ff0000ffULL;
    v = (v | (v << 8)) & 0x100f00f00f00f00fULL;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ULL;
    v = (v | (v << 2)) & 0x1249249249249249ULL;
    return v;
}

static inline uint64_t or_cell_coord(double v, double lo, double scale) {
    const double t = floor((v - lo) * scale);
    if (!(t > 0.0)) return 0;
    if (t >= 2097151.0) return 2097151;
    return (uint64_t)t;
}

void or_morton_keys(const double *x, const double *y, const double *z, int64_t n, const or_rootbox *rb,
                    uint64_t *keys) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        const uint64_t qx = or_cell_coord(x[i], rb->root_lo[0], rb->scale);
        const uint64_t qy = or_cell_coord(y[i], rb->root_lo[1], rb->scale);
        const uint64_t qz = or_cell_coord(z[i], rb->root_lo[2], rb->scale);
        keys[i] = (or_spread3(qx) << 2) | (or_spread3(qy) << 1) | or_spread3(qz);
    }
}

/* Stable LSD radix sort of (key, index), 8 passes of 8 bits over 63 bits. */
void or_sort_perm(const uint64_t *keys, int64_t n, int64_t *perm) {
    uint64_t *k0 = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(n ? n : 1));
    uint64_t *k1 = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(n ? n : 1));
    int64_t *p1 = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n ? n : 1));
    for (int64_t i = 0; i < n; ++i) { k0[i] = keys[i]; perm[i] = i; }
    int64_t *pa = perm, *pb = p1;
    uint64_t *ka = k0, *kb = k1;
    for (int pass = 0; pass < 8; ++pass) {
        const int sh = pass * 8;
        int64_t cnt[257];
        memset(cnt, 0, sizeof(cnt));
        for (int64_t i = 0; i < n; ++i) cnt[((ka[i] >> sh) & 0xff) + 1]++;
        for (int b = 0; b < 256; ++b) cnt[b + 1] += cnt[b];
        for (int64_t i = 0; i < n; ++i) {
            const int64_t d = cnt[(ka[i] >> sh) & 0xff]++;
            kb[d] = ka[i];
            pb[d] = pa[i];
        }
        uint64_t *tk = ka; ka = kb; kb = tk;
        int64_t *tp = pa; pa = pb; pb = tp;
    }
    /* 8 passes: result is back in perm / k0 */
    free(k0); free(k1); free(p1);
}

void or_reorder(or_system *s, const int64_t *perm) {
    const int64_t n = s->n;
    double *tmp = (double *)malloc(sizeof(double) * (size_t)(n ? n : 1));
    for (int f = 0; f < OR_NFIELD; ++f) {
        double *a = F(s, f);
        for (int64_t k = 0; k < n; ++k) tmp[k] = a[perm[k]];
        memcpy(a, tmp, sizeof(double) * (size_t)n);
    }
    free(tmp);
    int64_t *ti = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n ? n : 1));
    for (int64_t k = 0; k < n; ++k) ti[k] = s->id[perm[k]];
    memcpy(s->id, ti, sizeof(int64_t) * (size_t)n);
    free(ti);
    int32_t *tm = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n ? n : 1));
    for (int64_t k = 0; k < n; ++k) tm[k] = s->mat[perm[k]];
    memcpy(s->mat, tm, sizeof(int32_t) * (size_t)n);
    free(tm);
}

/* ------------------------------------------------------------------------ */
/* Octree over sorted keys                                                   */

static inline int or_digit(uint64_t key, int level) { return (int)((key >> (3 * (OR_KEY_LEVELS - level))) & 7); }

static int64_t or_new_cells(or_tree *t, int k) {
    if (t->n_cell + k > t->cap) {
        int64_t nc = t->cap * 2 + k + 16;
        or_cell *c = (or_cell *)realloc(t->c, sizeof(or_cell) * (size_t)nc);
        if (!c) return -1;
        t->c = c;
        t->cap = nc;
    }
    const int64_t at = t->n_cell;
    t->n_cell += k;
    return at;
}

static int or_split(or_tree *t, int64_t ci, const uint64_t *keys, int n_leaf) {
    const int32_t start = t->c[ci].start, count = t->c[ci].count, level = t->c[ci].level;
    t->c[ci].first_child = -1;
    t->c[ci].n_child = 0;
    if (count <= n_leaf || level >= OR_KEY_LEVELS) return 0;
    int32_t b[9];
    int32_t lo = start;
    for (int oct = 0; oct < 8; ++oct) {
        /* first index in [lo, start+count) whose digit at level+1 is >= oct */
        int32_t a = lo, len = start + count - lo;
        while (len > 0) {
            const int32_t half = len >> 1;
            if (or_digit(keys[a + half], level + 1) < oct) { a += half + 1; len -= half + 1; }
            else len = half;
        }
        b[oct] = a;
        lo = a;
    }
    b[8] = start + count;
    int nch = 0;
    for (int oct = 0; oct < 8; ++oct) nch += (b[oct + 1] > b[oct]);
    const int64_t first = or_new_cells(t, nch);
    if (first < 0) return -1;
    t->c[ci].first_child = (int32_t)first;
    t->c[ci].n_child = nch;
    int k = 0;
    for (int oct = 0; oct < 8; ++oct) {
        if (b[oct + 1] <= b[oct]) continue;
        or_cell *ch = &t->c[first + k];
        memset(ch, 0, sizeof(*ch));
        ch->start = b[oct];
        ch->count = b[oct + 1] - b[oct];
        ch->level = level + 1;
        ch->parent = (int32_t)ci;
        ++k;
    }
    for (k = 0; k < nch; ++k)
        if (or_split(t, first + k, keys, n_leaf) < 0) return -1;
    return 0;
}

int or_tree_build(or_tree *t, const double *x, const double *y, const double *z, const double *m,
                  const double *h, const uint64_t *keys, int64_t n, int n_leaf) {
    t->n_cell = 0;
    if (t->cap == 0) { t->cap = 1024; t->c = (or_cell *)malloc(sizeof(or_cell) * 1024); }
    const int64_t r = or_new_cells(t, 1);
    memset(&t->c[r], 0, sizeof(or_cell));
    t->c[r].start = 0;
    t->c[r].count = (int32_t)n;
    t->c[r].level = 0;
    t->c[r].parent = -1;
    if (or_split(t, r, keys, n_leaf) < 0) return -1;
    /* moments bottom-up: children always have larger indices than their parent */
    for (int64_t ci = t->n_cell - 1; ci >= 0; --ci) {
        or_cell *c = &t->c[ci];
        double mass = 0, mx = 0, my = 0, mz = 0, hm = 0;
        double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        if (c->n_child == 0) {
            for (int32_t j = c->start; j < c->start + c->count; ++j) {
                mass = mass + m[j];
                mx = mx + m[j] * x[j];
                my = my + m[j] * y[j];
                mz = mz + m[j] * z[j];
                if (h[j] > hm) hm = h[j];
                const double p[3] = {x[j], y[j], z[j]};
                for (int d = 0; d < 3; ++d) {
                    if (p[d] < lo[d]) lo[d] = p[d];
                    if (p[d] > hi[d]) hi[d] = p[d];
                }
            }
        } else {
            for (int k = 0; k < c->n_child; ++k) {
                const or_cell *ch = &t->c[c->first_child + k];
                mass = mass + ch->mass;
                mx = mx + ch->mx;
                my = my + ch->my;
                mz = mz + ch->mz;
                if (ch->hmax > hm) hm = ch->hmax;
                for (int d = 0; d < 3; ++d) {
                    if (ch->lo[d] < lo[d]) lo[d] = ch->lo[d];
                    if (ch->hi[d] > hi[d]) hi[d] = ch->hi[d];
                }
            }
        }
        c->mass = mass; c->mx = mx; c->my = my; c->mz = mz;
        c->com[0] = mx / mass; c->com[1] = my / mass; c->com[2] = mz / mass;
        c->hmax = hm;
        for (int d = 0; d < 3; ++d) { c->lo[d] = lo[d]; c->hi[d] = hi[d]; }
    }
    return 0;
}

void or_tree_free(or_tree *t) {
    free(t->c);
    free(t->keys);
    memset(t, 0, sizeof(*t));
}

/* i-groups: cells with count <= n_group whose parent has count > n_group, in key order */
static void or_groups_rec(const or_tree *t, int32_t ci, int n_group, int32_t *out, int64_t *k) {
    const or_cell *c = &t->c[ci];
    if (c->count <= n_group || c->n_child == 0) { out[(*k)++] = ci; return; }
    for (int j = 0; j < c->n_child; ++j) or_groups_rec(t, c->first_child + j, n_group, out, k);
}

int64_t or_tree_groups(const or_tree *t, int n_group, int32_t *group_cells) {
    int64_t k = 0;
    if (t->n_cell > 0 && t->c[0].count > 0) or_groups_rec(t, 0, n_group, group_cells, &k);
    return k;
}

/* squared distance from point p to the box [lo, hi]; zero inside */
static inline double or_dmin2(const double lo[3], const double hi[3], const double p[3]) {
    double d[3];
    for (int k = 0; k < 3; ++k) d[k] = (p[k] < lo[k]) ? (lo[k] - p[k]) : ((p[k] > hi[k]) ? (p[k] - hi[k]) : 0.0);
    return d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
}

/* ------------------------------------------------------------------------ */
/* SPH neighbour lists.  Gather (TreeForForceShort::Gather, main.cpp:79-80):
 * j is a neighbour of i iff |x_j - x_i|^2 < (2.5 h_i)^2.  Symmetric
 * (TreeForForceShort::Symmetry, main.cpp:81): iff |x_j - x_i|^2 <
 * (2.5 h_i)^2 or < (2.5 h_j)^2.  j = i is included.  Lists are ascending. */

typedef struct { int32_t *a; int64_t n, cap; } or_ibuf;

static void or_ibuf_push(or_ibuf *b, int32_t v) {
    if (b->n == b->cap) {
        b->cap = b->cap ? b->cap * 2 : 256;
        b->a = (int32_t *)realloc(b->a, sizeof(int32_t) * (size_t)b->cap);
    }
    b->a[b->n++] = v;
}

static void or_sph_walk(const or_tree *t, int32_t ci, const double *x, const double *y, const double *z,
                        const double *h, const double p[3], double H2, int mode, or_ibuf *out) {
    const or_cell *c = &t->c[ci];
    const double dm = or_dmin2(c->lo, c->hi, p);
    int visit = dm < H2;
    if (!visit && mode == 1) {
        const double Hc = OR_SUPPORT * c->hmax;
        visit = dm < Hc * Hc;
    }
    if (!visit) return;
    if (c->n_child == 0) {
        for (int32_t j = c->start; j < c->start + c->count; ++j) {
            const double dx = x[j] - p[0], dy = y[j] - p[1], dz = z[j] - p[2];
            const double r2 = dx * dx + dy * dy + dz * dz;
            int ok = r2 < H2;
            if (!ok && mode == 1) {
                const double Hj = OR_SUPPORT * h[j];
                ok = r2 < Hj * Hj;
            }
            if (ok) or_ibuf_push(out, j);
        }
        return;
    }
    for (int k = 0; k < c->n_child; ++k) or_sph_walk(t, c->first_child + k, x, y, z, h, p, H2, mode, out);
}

static void or_sph_collect(const or_tree *t, const double *x, const double *y, const double *z, const double *h,
                           int64_t i, int mode, or_ibuf *out) {
    out->n = 0;
    const double p[3] = {x[i], y[i], z[i]};
    const double H = OR_SUPPORT * h[i];
    if (t->n_cell > 0) or_sph_walk(t, 0, x, y, z, h, p, H * H, mode, out);
}

int64_t or_sph_list(const or_tree *t, const double *x, const double *y, const double *z, const double *h,
                    int64_t i, int mode, int32_t *out, int64_t cap) {
    or_ibuf b = {0, 0, 0};
    or_sph_collect(t, x, y, z, h, i, mode, &b);
    for (int64_t k = 0; k < b.n && k < cap; ++k) out[k] = b.a[k];
    const int64_t n = b.n;
    free(b.a);
    return n;
}

/* ------------------------------------------------------------------------ */
/* Gravity interaction lists (TreeForForceLong::Monopole, main.cpp:83,90).
 * A child cell is opened iff dmin^2(group box, child com) <= (child side /
 * theta)^2, i.e. rc2[level] = root_len^2/theta^2 * 0.25^level.  Cells are
 * opened breadth-first in FIFO order from the root: an opened leaf appends
 * its particles to EPJ (the group's own included); an opened internal cell
 * appends its unopened children to SPJ (monopoles) and its opened children
 * to the queue, both in octant order. */

typedef struct { or_ibuf epj, spj, queue; } or_glist;

static void or_grav_walk(const or_tree *t, int32_t root, const double blo[3], const double bhi[3],
                         const double *rc2, or_glist *L) {
    L->queue.n = 0;
    or_ibuf_push(&L->queue, root);
    for (int64_t head = 0; head < L->queue.n; ++head) {
        const or_cell *c = &t->c[L->queue.a[head]];
        if (c->n_child == 0) {
            for (int32_t j = c->start; j < c->start + c->count; ++j) or_ibuf_push(&L->epj, j);
            continue;
        }
        for (int k = 0; k < c->n_child; ++k) {
            const int32_t chi = c->first_child + k;
            const or_cell *ch = &t->c[chi];
            if (or_dmin2(blo, bhi, ch->com) <= rc2[ch->level]) or_ibuf_push(&L->queue, chi);
            else or_ibuf_push(&L->spj, chi);
        }
    }
}

static void or_rcrit_table(const or_tree *t, double theta, double rc2[OR_KEY_LEVELS + 1]) {
    rc2[0] = t->rb.root_len * t->rb.root_len / (theta * theta);
    for (int l = 1; l <= OR_KEY_LEVELS; ++l) rc2[l] = rc2[l - 1] * 0.25;
}

static void or_group_box(const double *x, const double *y, const double *z, int32_t start, int32_t count,
                         double lo[3], double hi[3]) {
    for (int d = 0; d < 3; ++d) { lo[d] = INFINITY; hi[d] = -INFINITY; }
    for (int32_t j = start; j < start + count; ++j) {
        const double p[3] = {x[j], y[j], z[j]};
        for (int d = 0; d < 3; ++d) {
            if (p[d] < lo[d]) lo[d] = p[d];
            if (p[d] > hi[d]) hi[d] = p[d];
        }
    }
}

int or_grav_list(const or_tree *t, const double *x, const double *y, const double *z, int32_t gcell,
                 double theta, int32_t *epj, int64_t cap_epj, int64_t *n_epj, int32_t *spj, int64_t cap_spj,
                 int64_t *n_spj) {
    double rc2[OR_KEY_LEVELS + 1];
    or_rcrit_table(t, theta, rc2);
    double lo[3], hi[3];
    or_group_box(x, y, z, t->c[gcell].start, t->c[gcell].count, lo, hi);
    or_glist L;
    memset(&L, 0, sizeof(L));
    or_grav_walk(t, 0, lo, hi, rc2, &L);
    for (int64_t k = 0; k < L.epj.n && k < cap_epj; ++k) epj[k] = L.epj.a[k];
    for (int64_t k = 0; k < L.spj.n && k < cap_spj; ++k) spj[k] = L.spj.a[k];
    *n_epj = L.epj.n;
    *n_spj = L.spj.n;
    free(L.epj.a);
    free(L.spj.a);
    free(L.queue.a);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Passes                                                                     */

/* CalcDensity, force.h:9-23 (gather list; write-back as RealPtcl::copyFromForce, class.h:127-130) */
void or_pass_density(or_system *s, const or_tree *t, const or_config *cfg) {
    (void)cfg;
    const int64_t n = s->n;
    const double *x = F(s, OR_X), *y = F(s, OR_Y), *z = F(s, OR_Z), *m = F(s, OR_MASS);
    double *h = F(s, OR_SMTH), *dens = F(s, OR_DENS);
    double *nd = (double *)malloc(sizeof(double) * (size_t)(n ? n : 1));
    double *nh = (double *)malloc(sizeof(double) * (size_t)(n ? n : 1));
#pragma omp parallel
    {
        or_ibuf b = {0, 0, 0};
#pragma omp for schedule(dynamic, 64)
        for (int64_t i = 0; i < n; ++i) {
            or_sph_collect(t, x, y, z, h, i, 0, &b);
            double d = 0.0;
            for (int64_t k = 0; k < b.n; ++k) {
                const int32_t j = b.a[k];
                d += m[j] * or_kernel_W(x[j] - x[i], y[j] - y[i], z[j] - z[i], h[i]);
            }
            d = or_max(OR_DENS_FLOOR, d);
            nd[i] = d;
            nh[i] = OR_SMTH_COEF * pow(m[i] / d, 1.0 / 3.0);
        }
        free(b.a);
    }
    memcpy(dens, nd, sizeof(double) * (size_t)n);
    memcpy(h, nh, sizeof(double) * (size_t)n);
    free(nd);
    free(nh);
}

/* CalcPressure, force.h:26-32 */
void or_pass_pressure(or_system *s, const or_config *cfg) {
    const int64_t n = s->n;
    double *dens = F(s, OR_DENS), *eng = F(s, OR_ENG), *P = F(s, OR_PRES), *cs = F(s, OR_SNDS);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) or_eos_eval(&cfg->mat[s->mat[i]], dens[i], eng[i], &P[i], &cs[i]);
}

/* CalcDerivative, force.h:89-106, then RealPtcl::copyFromForce(Drvt) with the
 * Balsara switch, class.h:132-142 */
void or_pass_derivative(or_system *s, const or_tree *t) {
    const int64_t n = s->n;
    const double *x = F(s, OR_X), *y = F(s, OR_Y), *z = F(s, OR_Z), *m = F(s, OR_MASS), *h = F(s, OR_SMTH);
    const double *vx = F(s, OR_VX), *vy = F(s, OR_VY), *vz = F(s, OR_VZ), *dens = F(s, OR_DENS),
                 *cs = F(s, OR_SNDS);
    double *divv = F(s, OR_DIVV), *rx = F(s, OR_ROTX), *ry = F(s, OR_ROTY), *rz = F(s, OR_ROTZ),
           *gh = F(s, OR_GRADH), *bal = F(s, OR_BAL);
#pragma omp parallel
    {
        or_ibuf b = {0, 0, 0};
#pragma omp for schedule(dynamic, 64)
        for (int64_t i = 0; i < n; ++i) {
            or_sph_collect(t, x, y, z, h, i, 0, &b);
            double dv_ = 0.0, r0 = 0.0, r1 = 0.0, r2 = 0.0, gs = 0.0;
            for (int64_t k = 0; k < b.n; ++k) {
                const int32_t j = b.a[k];
                const double dx = x[i] - x[j], dy = y[i] - y[j], dz = z[i] - z[j];
                const double ux = vx[i] - vx[j], uy = vy[i] - vy[j], uz = vz[i] - vz[j];
                double g[3];
                or_kernel_gradW(dx, dy, dz, h[i], g);
                const double W = or_kernel_W(dx, dy, dz, h[i]);
                const double ax = -m[j] * ux, ay = -m[j] * uy, az = -m[j] * uz;
                dv_ += or_dot(ax, ay, az, g[0], g[1], g[2]);
                r0 += ay * g[2] - az * g[1];
                r1 += az * g[0] - ax * g[2];
                r2 += ax * g[1] - ay * g[0];
                gs -= m[j] / h[i] * (3 * W + or_dot(dx, dy, dz, g[0], g[1], g[2]));
            }
            gs = 1.0 / (1.0 + h[i] * gs / (3 * dens[i]));
            dv_ /= dens[i];
            r0 /= dens[i];
            r1 /= dens[i];
            r2 /= dens[i];
            divv[i] = dv_;
            rx[i] = r0; ry[i] = r1; rz[i] = r2;
            gh[i] = gs;
            bal[i] = fabs(dv_) / (fabs(dv_) + sqrt(or_dot(r0, r1, r2, r0, r1, r2)) + 1.0e-4 * cs[i] / h[i]);
        }
        free(b.a);
    }
}

/* CalcHydroForce, force.h:113-147 (symmetric list; v_sig_max over the true
 * symmetric neighbour set), write-back class.h:144-148 */
void or_pass_hydro(or_system *s, const or_tree *t) {
    const int64_t n = s->n;
    const double *x = F(s, OR_X), *y = F(s, OR_Y), *z = F(s, OR_Z), *m = F(s, OR_MASS), *h = F(s, OR_SMTH);
    const double *vx = F(s, OR_VX), *vy = F(s, OR_VY), *vz = F(s, OR_VZ), *dens = F(s, OR_DENS);
    const double *P = F(s, OR_PRES), *cs = F(s, OR_SNDS), *gh = F(s, OR_GRADH), *bal = F(s, OR_BAL);
    double *ax = F(s, OR_AX), *ay = F(s, OR_AY), *az = F(s, OR_AZ), *ed = F(s, OR_ENGDOT), *dt = F(s, OR_DT);
#pragma omp parallel
    {
        or_ibuf b = {0, 0, 0};
#pragma omp for schedule(dynamic, 64)
        for (int64_t i = 0; i < n; ++i) {
            or_sph_collect(t, x, y, z, h, i, 1, &b);
            double a0 = 0, a1 = 0, a2 = 0, e = 0, vmax = 0.0;
            const double Ai = gh[i] * P[i] / (dens[i] * dens[i]);
            for (int64_t k = 0; k < b.n; ++k) {
                const int32_t j = b.a[k];
                const double dx = x[i] - x[j], dy = y[i] - y[j], dz = z[i] - z[j];
                const double ux = vx[i] - vx[j], uy = vy[i] - vy[j], uz = vz[i] - vz[j];
                const double dvdr = or_dot(ux, uy, uz, dx, dy, dz);
                const double w = (dvdr < 0) ? dvdr / sqrt(or_dot(dx, dy, dz, dx, dy, dz)) : 0;
                const double vsig = cs[i] + cs[j] - 3.0 * w;
                vmax = or_max(vmax, vsig);
                const double AV = -OR_AV_STRENGTH * 0.5 * vsig * w / (0.5 * (dens[i] + dens[j])) * 0.5 *
                                  (bal[i] + bal[j]);
                double gi[3], gj[3];
                or_kernel_gradW(dx, dy, dz, h[i], gi);
                or_kernel_gradW(dx, dy, dz, h[j], gj);
                const double gw0 = 0.5 * (gi[0] * gh[i] + gj[0] * gh[j]);
                const double gw1 = 0.5 * (gi[1] * gh[i] + gj[1] * gh[j]);
                const double gw2 = 0.5 * (gi[2] * gh[i] + gj[2] * gh[j]);
                const double Aj = gh[j] * P[j] / (dens[j] * dens[j]);
                a0 -= m[j] * (Ai * gi[0] + Aj * gj[0] + AV * gw0);
                a1 -= m[j] * (Ai * gi[1] + Aj * gj[1] + AV * gw1);
                a2 -= m[j] * (Ai * gi[2] + Aj * gj[2] + AV * gw2);
                const double c = m[j] * (Ai + 0.5 * AV);
                e += or_dot(c * ux, c * uy, c * uz, gw0, gw1, gw2);
            }
            ax[i] = a0; ay[i] = a1; az[i] = a2;
            ed[i] = e;
            dt[i] = OR_CFL * 2.0 * h[i] / vmax;
        }
        free(b.a);
    }
}

/* CalcGravityForce<EPJ::Grav> then CalcGravityForce<SPJMonopole>, force.h:154-168,
 * eps^2 = h^2 (class.h:336); write-back class.h:150-154 */
void or_pass_gravity(or_system *s, const or_tree *t, const or_config *cfg) {
    const int64_t n = s->n;
    const double *x = F(s, OR_X), *y = F(s, OR_Y), *z = F(s, OR_Z), *m = F(s, OR_MASS), *h = F(s, OR_SMTH);
    double *gx = F(s, OR_GX), *gy = F(s, OR_GY), *gz = F(s, OR_GZ), *pot = F(s, OR_POT);
    const double G = cfg->G;
    int32_t *groups = (int32_t *)malloc(sizeof(int32_t) * (size_t)(t->n_cell ? t->n_cell : 1));
    const int64_t ng = or_tree_groups(t, cfg->n_group, groups);
    double rc2[OR_KEY_LEVELS + 1];
    or_rcrit_table(t, cfg->theta, rc2);
#pragma omp parallel
    {
        or_glist L;
        memset(&L, 0, sizeof(L));
#pragma omp for schedule(dynamic, 1)
        for (int64_t g = 0; g < ng; ++g) {
            const or_cell *gc = &t->c[groups[g]];
            double lo[3], hi[3];
            or_group_box(x, y, z, gc->start, gc->count, lo, hi);
            L.epj.n = 0;
            L.spj.n = 0;
            or_grav_walk(t, 0, lo, hi, rc2, &L);
            for (int32_t i = gc->start; i < gc->start + gc->count; ++i) {
                const double eps2 = h[i] * h[i];
                double a0 = 0, a1 = 0, a2 = 0, p = 0;
                for (int64_t k = 0; k < L.epj.n; ++k) {
                    const int32_t j = L.epj.a[k];
                    const double dx = x[i] - x[j], dy = y[i] - y[j], dz = z[i] - z[j];
                    const double dr2 = or_dot(dx, dy, dz, dx, dy, dz);
                    const double dri = 1.0 / sqrt(dr2 + eps2);
                    const double mdr3 = m[j] * (dri * dri * dri);
                    a0 -= G * mdr3 * dx;
                    a1 -= G * mdr3 * dy;
                    a2 -= G * mdr3 * dz;
                    p -= G * m[j] * dri;
                }
                for (int64_t k = 0; k < L.spj.n; ++k) {
                    const or_cell *c = &t->c[L.spj.a[k]];
                    const double dx = x[i] - c->com[0], dy = y[i] - c->com[1], dz = z[i] - c->com[2];
                    const double dr2 = or_dot(dx, dy, dz, dx, dy, dz);
                    const double dri = 1.0 / sqrt(dr2 + eps2);
                    const double mdr3 = c->mass * (dri * dri * dri);
                    a0 -= G * mdr3 * dx;
                    a1 -= G * mdr3 * dy;
                    a2 -= G * mdr3 * dz;
                    p -= G * c->mass * dri;
                }
                gx[i] = a0; gy[i] = a1; gz[i] = a2; pot[i] = p;
            }
        }
        free(L.epj.a);
        free(L.spj.a);
        free(L.queue.a);
    }
    free(groups);
}

/* getTimeStepGlobal, integral.h:4-20 (the acceleration criterion is computed but unused there) */
double or_dt_global(const or_system *s) {
    const double *dt = s->F + (int64_t)OR_DT * s->n;
    double r = 1.0e+30;
    for (int64_t i = 0; i < s->n; ++i) r = or_min(r, or_min(dt[i], 1.0e+30));
    return r;
}

/* GI_universal::addExternalForce, GI.h:458-465 */
static void or_ext_force(or_system *s, const or_config *cfg) {
    if (!cfg->ext_damp || s->time >= cfg->ext_damp_tend) return;
    const int64_t n = s->n;
    double *ax = F(s, OR_AX), *ay = F(s, OR_AY), *az = F(s, OR_AZ);
    const double *vx = F(s, OR_VX), *vy = F(s, OR_VY), *vz = F(s, OR_VZ), *dt = F(s, OR_DT);
    for (int64_t i = 0; i < n; ++i) {
        ax[i] += -vx[i] * 0.05 / dt[i];
        ay[i] += -vy[i] * 0.05 / dt[i];
        az[i] += -vz[i] * 0.05 / dt[i];
    }
}

/* ------------------------------------------------------------------------ */
/* Step                                                                       */

static int or_sort_and_build(or_system *s, or_tree *t, int n_leaf) {
    const int64_t n = s->n;
    or_root_box(F(s, OR_X), F(s, OR_Y), F(s, OR_Z), n, &t->rb);
    uint64_t *keys = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(n ? n : 1));
    int64_t *perm = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n ? n : 1));
    or_morton_keys(F(s, OR_X), F(s, OR_Y), F(s, OR_Z), n, &t->rb, keys);
    or_sort_perm(keys, n, perm);
    or_reorder(s, perm);
    uint64_t *sk = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(n ? n : 1));
    for (int64_t k = 0; k < n; ++k) sk[k] = keys[perm[k]];
    free(keys);
    free(perm);
    free(t->keys);
    t->keys = sk;
    return or_tree_build(t, F(s, OR_X), F(s, OR_Y), F(s, OR_Z), F(s, OR_MASS), F(s, OR_SMTH), sk, n, n_leaf);
}

int or_sort_system(or_system *s, or_tree *t, int n_leaf) { return or_sort_and_build(s, t, n_leaf); }

/* refresh cell bounding boxes / hmax after h changed (positions unchanged) */
static void or_tree_refresh_h(or_tree *t, const double *h) {
    for (int64_t ci = t->n_cell - 1; ci >= 0; --ci) {
        or_cell *c = &t->c[ci];
        double hm = 0;
        if (c->n_child == 0) {
            for (int32_t j = c->start; j < c->start + c->count; ++j)
                if (h[j] > hm) hm = h[j];
        } else {
            for (int k = 0; k < c->n_child; ++k)
                if (t->c[c->first_child + k].hmax > hm) hm = t->c[c->first_child + k].hmax;
        }
        c->hmax = hm;
    }
}

/* main.cpp:138-146: density x4, pressure, derivative, hydro, gravity */
int or_compute_forces(or_system *s, const or_config *cfg) {
    or_tree t;
    memset(&t, 0, sizeof(t));
    if (or_sort_and_build(s, &t, cfg->n_leaf) < 0) { or_tree_free(&t); return -1; }
    for (int it = 0; it < cfg->n_dens_iter; ++it) or_pass_density(s, &t, cfg);
    or_tree_refresh_h(&t, F(s, OR_SMTH));
    or_pass_pressure(s, cfg);
    or_pass_derivative(s, &t);
    or_pass_hydro(s, &t);
    if (cfg->self_gravity) or_pass_gravity(s, &t, cfg);
    or_tree_free(&t);
    return 0;
}

/* RealPtcl::initialize, class.h:196-199 */
int or_initialize_smth(or_system *s) {
    double *h = F(s, OR_SMTH), *gh = F(s, OR_GRADH);
    const double *m = F(s, OR_MASS), *d = F(s, OR_DENS);
    for (int64_t i = 0; i < s->n; ++i) {
        h[i] = OR_SMTH_COEF * pow(m[i] / d[i], 1.0 / 3.0);
        gh[i] = 1.0;
    }
    return 0;
}

/* main.cpp:92-105 */
int or_prologue(or_system *s, const or_config *cfg) {
    if (or_compute_forces(s, cfg) < 0) return -1;
    s->dt = or_dt_global(s);
    or_ext_force(s, cfg);
    return 0;
}

/* main.cpp:125-173 loop body (mode 1; output and mode-2 entropy path excluded) */
/* initialKick, fullDrift, predict: class.h:201-219 (FLAG_R00 is false, so AVa is not evolved) */
void or_kick_drift_predict(or_system *s, double dt) {
    const int64_t n = s->n;
    double *x = F(s, OR_X), *y = F(s, OR_Y), *z = F(s, OR_Z);
    double *vx = F(s, OR_VX), *vy = F(s, OR_VY), *vz = F(s, OR_VZ);
    const double *ax = F(s, OR_AX), *ay = F(s, OR_AY), *az = F(s, OR_AZ);
    const double *gx = F(s, OR_GX), *gy = F(s, OR_GY), *gz = F(s, OR_GZ);
    double *hx = F(s, OR_VHX), *hy = F(s, OR_VHY), *hz = F(s, OR_VHZ);
    double *u = F(s, OR_ENG), *uh = F(s, OR_ENGHALF);
    const double *ud = F(s, OR_ENGDOT);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        hx[i] = vx[i] + 0.5 * dt * (ax[i] + gx[i]);
        hy[i] = vy[i] + 0.5 * dt * (ay[i] + gy[i]);
        hz[i] = vz[i] + 0.5 * dt * (az[i] + gz[i]);
        uh[i] = u[i] + 0.5 * dt * ud[i];
        x[i] += dt * hx[i];
        y[i] += dt * hy[i];
        z[i] += dt * hz[i];
        vx[i] += dt * (ax[i] + gx[i]);
        vy[i] += dt * (ay[i] + gy[i]);
        vz[i] += dt * (az[i] + gz[i]);
        u[i] += dt * ud[i];
    }
}

/* finalKick, dampMotion: class.h:221-229 */
void or_final_kick(or_system *s, double dt, double damp) {
    const int64_t n = s->n;
    double *vx = F(s, OR_VX), *vy = F(s, OR_VY), *vz = F(s, OR_VZ);
    const double *ax = F(s, OR_AX), *ay = F(s, OR_AY), *az = F(s, OR_AZ);
    const double *gx = F(s, OR_GX), *gy = F(s, OR_GY), *gz = F(s, OR_GZ);
    const double *hx = F(s, OR_VHX), *hy = F(s, OR_VHY), *hz = F(s, OR_VHZ);
    double *u = F(s, OR_ENG);
    const double *ud = F(s, OR_ENGDOT), *uh = F(s, OR_ENGHALF);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        vx[i] = hx[i] + 0.5 * dt * (ax[i] + gx[i]);
        vy[i] = hy[i] + 0.5 * dt * (ay[i] + gy[i]);
        vz[i] = hz[i] + 0.5 * dt * (az[i] + gz[i]);
        u[i] = uh[i] + 0.5 * dt * ud[i];
        vx[i] *= damp;
        vy[i] *= damp;
        vz[i] *= damp;
    }
}

/* main.cpp:125-173 loop body (output excluded); returns -2 when a mode-2
 * lookup is undefined or non-finite */
int or_step(or_system *s, const or_config *cfg, int n_steps) {
    for (int st = 0; st < n_steps; ++st) {
        const double dt = s->dt;
        or_kick_drift_predict(s, dt);
        s->time += dt;
        if (or_compute_forces(s, cfg) < 0) return -1;
        or_ext_force(s, cfg);
        or_final_kick(s, dt, cfg->damping);
        if (cfg->mode == 2 && or_entropy_step(s, cfg) > 0) return -2;   /* main.cpp:155-158 */
        s->dt = or_dt_global(s);
        s->step += 1;
    }
    return 0;
}
