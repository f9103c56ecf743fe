/* CPU oracle for the FDPS_SPH per-step interaction path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's
 * algorithm (src/force.h, src/kernel.h, src/EoS.h, src/interpolation.h,
 * src/class.h, src/integral.h, src/main.cpp:92-173) plus an explicit
 * restatement of the tree / group / interaction-list semantics that FDPS
 * v5.0c provides to the reference (FDPS is not vendored with the reference,
 * so those semantics are this project's written specification).  It is used
 * by the tests as the checker and by bench.py as the CPU baseline; the
 * product library never links or calls it.
 *
 * Parity status: pair arithmetic, EoS lookup, Balsara switch, integrator and
 * global dt are pinned against the reference's own code (compiled from its
 * headers by oracle/ref, golden vectors in tests/golden).  Tree, group and
 * list membership are "parity unpinned" against FDPS itself (absent); they
 * are pinned only against this restatement.
 */
#ifndef SPH_ORACLE_H
#define SPH_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Field-major particle block: field f of particle i is F[f * n + i]. */
enum or_field {
    OR_X = 0, OR_Y, OR_Z, OR_VX, OR_VY, OR_VZ, OR_MASS, OR_SMTH, OR_DENS, OR_ENG,
    OR_PRES, OR_SNDS, OR_DIVV, OR_ROTX, OR_ROTY, OR_ROTZ, OR_BAL, OR_AVA, OR_GRADH,
    OR_AX, OR_AY, OR_AZ, OR_ENGDOT, OR_VHX, OR_VHY, OR_VHZ, OR_ENGHALF, OR_DT,
    OR_GX, OR_GY, OR_GZ, OR_POT, OR_ENT, OR_TEMP, OR_NFIELD
};

typedef struct {
    int32_t kind;          /* 0 = rho-u table (BilinearInterpolation), 1 = analytic Tillotson, 2 = ideal gas */
    int32_t n_rho, n_u;    /* table extents */
    const double *rho;     /* [n_rho] density axis, ascending */
    const double *u;       /* [n_u]   energy axis, ascending  */
    const double *pres;    /* [n_rho * n_u], rho-major */
    const double *snds;    /* [n_rho * n_u] */
    double par[10];        /* Tillotson: rho0 u0 uiv ucv A B a b alpha beta; ideal gas: par[0] = gamma */
    const double *temp;    /* [n_rho * n_u] column 2 (NULL: no mode-2 data) */
    const double *ent;     /* [n_rho * n_u] column 5: the reference's full_entropies */
    const double *line_rho;/* [n_rho * n_u] column 0 of every line: full_densities */
    const double *line_u;  /* [n_rho * n_u] column 1 of every line: full_energies */
} or_material;

typedef struct {
    double theta;          /* gravity opening angle (FDPS default for the reference: 0.5, main.cpp:90) */
    int32_t n_leaf;        /* leaf limit of the octree (8, main.cpp:90) */
    int32_t n_group;       /* gravity i-group limit (256, main.cpp:90) */
    int32_t n_dens_iter;   /* density / smoothing-length passes (4, param.h:11 + main.cpp:138) */
    int32_t self_gravity;  /* SELF_GRAVITY (GI.h:4) */
    int32_t ext_damp;      /* GI_universal::addExternalForce (GI.h:458-465) on/off */
    double ext_damp_tend;  /* 5000 s in the reference */
    double damping;        /* dampMotion factor (GI.h:62 "damping", default 1) */
    double G;              /* 6.67e-11 (force.h:171-172) */
    int32_t n_mat;
    const or_material *mat;
    int32_t mode;          /* 1 or 2 (main.cpp:115, 155-158) */
    int32_t entropy_grid;  /* grid_length (120, EoS.h:250-251, 403-404) */
    int32_t entropy_abs;   /* 0: int abs(int) of the truncated distance, 1: fabs */
    double mantle_entropy, core_entropy;   /* main.cpp:116-119 */
} or_config;

typedef struct {
    int64_t n;
    double *F;             /* [OR_NFIELD * n] */
    int64_t *id;           /* [n] */
    int32_t *mat;          /* [n] material index */
    double time, dt;       /* system_t (class.h:8-14) */
    int64_t step;
} or_system;

/* --- pair arithmetic (kernel.h, force.h) -------------------------------- */
double or_kernel_W(double dx, double dy, double dz, double h);
void or_kernel_gradW(double dx, double dy, double dz, double h, double g[3]);

/* --- EoS ---------------------------------------------------------------- */
double or_table_lookup(const double *rho_ax, int n_rho, const double *u_ax, int n_u, const double *plane,
                       double rho, double u);
void or_eos_eval(const or_material *m, double rho, double u, double *P, double *cs);
/* EoS_t::Temperature / Entropy (bilinear on columns 2 / 5) and InternalEnergy
 * (RestrictedBilinearInterpolation over every table line, literal O(lines)
 * scans); *undef = 1 where the reference would index outside its vectors
 * (the result is then NaN). */
double or_eos_temperature(const or_material *m, double rho, double u);
double or_eos_entropy(const or_material *m, double rho, double u);
double or_eos_internal_energy(const or_material *m, double rho, double s, int grid, int abs_mode, int *undef);
/* SetConstantEntropy + CalcAll (force.h:55-84) over the system; returns the
 * number of undefined or non-finite lookups. */
int64_t or_entropy_step(or_system *s, const or_config *cfg);

/* --- tree --------------------------------------------------------------- */
typedef struct {
    double root_lo[3];
    double root_len;
    double scale;          /* 2^21 / root_len */
} or_rootbox;

void or_root_box(const double *x, const double *y, const double *z, int64_t n, or_rootbox *rb);
void or_morton_keys(const double *x, const double *y, const double *z, int64_t n, const or_rootbox *rb,
                    uint64_t *keys);
/* stable ascending order of keys: perm[k] = index of the k-th smallest */
void or_sort_perm(const uint64_t *keys, int64_t n, int64_t *perm);

typedef struct {
    int32_t start, count, level, first_child, n_child, parent;
    double mass, mx, my, mz;   /* monopole moments */
    double com[3];
    double lo[3], hi[3];       /* particle bounding box */
    double hmax;
} or_cell;

typedef struct {
    int64_t n_cell, cap;
    or_cell *c;
    or_rootbox rb;
    uint64_t *keys;            /* sorted keys [n] */
} or_tree;

/* Builds the octree over particles that are already in ascending key order. */
int or_tree_build(or_tree *t, const double *x, const double *y, const double *z, const double *m,
                  const double *h, const uint64_t *sorted_keys, int64_t n, int n_leaf);
void or_tree_free(or_tree *t);
int64_t or_tree_groups(const or_tree *t, int n_group, int32_t *group_cells /* [n_cell] */);

/* --- lists -------------------------------------------------------------- */
/* SPH neighbour list of particle i: mode 0 = gather (r2 < H_i^2), 1 = symmetric (r2 < max(H_i,H_j)^2).
   Writes ascending j into out (capacity cap), returns the count (may exceed cap). */
int64_t or_sph_list(const or_tree *t, const double *x, const double *y, const double *z, const double *h,
                    int64_t i, int mode, int32_t *out, int64_t cap);
/* Gravity interaction list of group g (cell index gcell): EPJ particle indices (ascending) and SPJ cell
   indices (walk order).  Returns 0; counts via n_epj / n_spj (may exceed caps). */
int or_grav_list(const or_tree *t, const double *x, const double *y, const double *z, int32_t gcell,
                 double theta, int32_t *epj, int64_t cap_epj, int64_t *n_epj, int32_t *spj, int64_t cap_spj,
                 int64_t *n_spj);

/* --- passes over a sorted system (tree already built) ------------------- */
void or_pass_density(or_system *s, const or_tree *t, const or_config *cfg);
void or_pass_pressure(or_system *s, const or_config *cfg);
void or_pass_derivative(or_system *s, const or_tree *t);
void or_pass_hydro(or_system *s, const or_tree *t);
void or_pass_gravity(or_system *s, const or_tree *t, const or_config *cfg);
double or_dt_global(const or_system *s);

/* --- whole step (main.cpp:92-173) --------------------------------------- */
/* Sorts the system by Morton key (stable), rebuilds the tree and evaluates all passes. */
int or_compute_forces(or_system *s, const or_config *cfg);
int or_initialize_smth(or_system *s);      /* RealPtcl::initialize (class.h:196-199) */
int or_prologue(or_system *s, const or_config *cfg);   /* main.cpp:92-105 */
int or_step(or_system *s, const or_config *cfg, int n_steps);  /* main.cpp:125-173 loop body */

void or_kick_drift_predict(or_system *s, double dt);          /* class.h:201-219 */
void or_final_kick(or_system *s, double dt, double damping);   /* class.h:221-229 */

/* helpers used by tests */
void or_reorder(or_system *s, const int64_t *perm);
int or_sort_system(or_system *s, or_tree *t, int n_leaf);   /* keys + stable sort + reorder + tree build */
int or_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
