/* sph_gb300.h -- C ABI of the GB300 implementation of FDPS_SPH's per-step
 * interaction path (libsph_gb300.so).
 *
 * Two families of entry points:
 *
 *  1. Functor-compatible batch calls.  They take the reference's own
 *     interaction payloads (src/class.h EPI/EPJ/RESULT layouts, all F64/S64)
 *     and apply exactly the reference functor (src/force.h) to every "walk"
 *     (one i-group with its j-list), the way FDPS's
 *     calcForceAllAndWriteBackMultiWalk drives a dispatch / retrieve pair.
 *     They replace the CPU loops inside
 *       STD::CalcDensity::operator()      force.h:9-23
 *       STD::CalcDerivative::operator()   force.h:89-106
 *       STD::CalcHydroForce::operator()   force.h:113-147
 *       STD::CalcGravityForce<T>::operator() force.h:154-168 (EPJ then SPJ)
 *     at the call sites main.cpp:93,97,98,100-101,139,142,143,145-146.
 *
 *  2. Device-resident whole-pass calls.  Particle state lives in HBM; the
 *     library builds the Morton-key octree, neighbour and interaction lists
 *     on the device and runs the complete step of main.cpp:125-173
 *     (kick-drift-predict, density x4, EoS, derivative + Balsara, hydro,
 *     tree gravity, final kick, global dt).
 *
 * Every entry point returns an int status: SPH_OK (0) or a negative error
 * code; sph_last_error() gives a message.  No C++ exception crosses the ABI.
 * A context is used by one host thread at a time; different contexts are
 * independent.
 */
#ifndef SPH_GB300_H
#define SPH_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define SPH_OK 0
#define SPH_ERR_ARG (-1)        /* bad argument (null pointer, negative size, unknown material ...) */
#define SPH_ERR_CUDA (-2)       /* a CUDA runtime call failed */
#define SPH_ERR_OOM (-3)        /* device or pinned allocation failed */
#define SPH_ERR_TABLE (-4)      /* EoS table missing, malformed or not ascending */
#define SPH_ERR_NONFINITE (-5)  /* non-finite state detected (positions, density, dt) */
#define SPH_ERR_CAPACITY (-6)   /* a list or tree capacity was exceeded and could not be grown */
#define SPH_ERR_STATE (-7)      /* call out of order (e.g. step before upload) */
#define SPH_ERR_TIMEOUT (-8)    /* a bounded device wait gave up */

/* ---- reference interaction payloads (src/class.h) ------------------------ */
typedef struct { double pos[3]; double mass; double smth; int64_t id; } sph_epi_dens;        /* class.h:233-258, 48 B */
typedef struct { double mass; double pos[3]; double smth; } sph_epj_dens;                    /* class.h:342-365, 40 B */
typedef struct { double dens; double smth; } sph_result_dens;                                /* class.h:36-44, 16 B */

typedef struct { double pos[3]; double vel[3]; double smth; double dens; } sph_epi_drvt;     /* class.h:260-281, 64 B */
typedef struct { double mass; double pos[3]; double vel[3]; double smth; } sph_epj_drvt;     /* class.h:367-392, 64 B */
typedef struct { double div_v; double rot_v[3]; double grad_smth; } sph_result_drvt;         /* class.h:47-58, 40 B */

typedef struct {
    double pos[3]; double vel[3]; double smth; double dens; double pres; double snds;
    double grad_smth; double Bal; double AVa; int64_t id;
} sph_epi_hydro;                                                                             /* class.h:283-315, 112 B */
typedef struct {
    double pos[3]; double vel[3]; double dens; double mass; double smth; double pres;
    double grad_smth; double snds; double Bal; double AVa; int64_t id;
} sph_epj_hydro;                                                                             /* class.h:394-432, 120 B */
typedef struct { double acc[3]; double eng_dot; double dt; } sph_result_hydro;              /* class.h:61-72, 40 B */

typedef struct { double pos[3]; double eps2; int64_t id; } sph_epi_grav;                     /* class.h:317-338, 40 B */
typedef struct { double pos[3]; double mass; int64_t id; } sph_epj_grav;                     /* class.h:434-453, 40 B */
typedef struct { double mass; double pos[3]; } sph_spj_monopole;                             /* FDPS SPJMonopole, 32 B */
typedef struct { double acc[3]; double pot; double dt; } sph_result_grav;                    /* class.h:75-86, 40 B */

/* ---- 1. functor-compatible batch entry points ----------------------------
 * dispatch: moves the walks to the device (sph_batch_set_staging) and
 * launches asynchronously on the stream of `tag` (0 <= tag < 64); it returns
 * once it has read the caller's arrays.  retrieve: waits for that stream and
 * writes result[w][0..n_epi[w]) for every walk (n_epi as dispatched).  Results
 * are the reference functor's: RESULT::clear() (class.h:41-85) followed by
 * the i x j loop over the walk's full j-list.  Return 0 on success, as
 * FDPS's dispatch / retrieve callbacks do.  The signatures are those of the
 * callbacks calcForceAllAndWriteBackMultiWalk takes for short-range
 * (dens, drvt, hydro) and long-range (grav) trees. */
int sph_dispatch_dens(int tag, int n_walk, const sph_epi_dens **epi, const int *n_epi,
                      const sph_epj_dens **epj, const int *n_epj);
int sph_retrieve_dens(int tag, int n_walk, const int *n_epi, sph_result_dens **result);
int sph_dispatch_drvt(int tag, int n_walk, const sph_epi_drvt **epi, const int *n_epi,
                      const sph_epj_drvt **epj, const int *n_epj);
int sph_retrieve_drvt(int tag, int n_walk, const int *n_epi, sph_result_drvt **result);
int sph_dispatch_hydro(int tag, int n_walk, const sph_epi_hydro **epi, const int *n_epi,
                       const sph_epj_hydro **epj, const int *n_epj);
int sph_retrieve_hydro(int tag, int n_walk, const int *n_epi, sph_result_hydro **result);
int sph_dispatch_grav(int tag, int n_walk, const sph_epi_grav **epi, const int *n_epi,
                      const sph_epj_grav **epj, const int *n_epj,
                      const sph_spj_monopole **spj, const int *n_spj);
int sph_retrieve_grav(int tag, int n_walk, const int *n_epi, sph_result_grav **result);
/* Index form: the dispatch callbacks of calcForceAllAndWriteBackMultiWalkIndex, retrieved with
 * the sph_retrieve_* above.  A call with send_flag != 0 first copies the pass's whole EPJ array
 * (epj[0..n_epj_tot)) and, for gravity, SPJ array to the device, where they stay for the kind's
 * later index dispatches (FDPS sends them once per pass, with n_walk = 0); it waits for index
 * dispatches of the same kind already issued, so it must not overlap new ones issued from other
 * threads.  The walks then carry indices: walk w's j entries are epj[id_epj[w][k]], k <
 * n_epj[w] (and spj[id_spj[w][k]]), in that order, so each j crosses the host link once per pass
 * instead of once per walk that lists it.  Index walks before a send fail with SPH_ERR_STATE; an
 * index outside the sent array makes the retrieve fail with SPH_ERR_ARG (the kernel reads entry
 * 0 in its place).  Results equal the payload form's bit for bit. */
int sph_dispatch_index_dens(int tag, int n_walk, const sph_epi_dens **epi, const int *n_epi, const int **id_epj,
                            const int *n_epj, const sph_epj_dens *epj, int n_epj_tot, int send_flag);
int sph_dispatch_index_drvt(int tag, int n_walk, const sph_epi_drvt **epi, const int *n_epi, const int **id_epj,
                            const int *n_epj, const sph_epj_drvt *epj, int n_epj_tot, int send_flag);
int sph_dispatch_index_hydro(int tag, int n_walk, const sph_epi_hydro **epi, const int *n_epi, const int **id_epj,
                             const int *n_epj, const sph_epj_hydro *epj, int n_epj_tot, int send_flag);
int sph_dispatch_index_grav(int tag, int n_walk, const sph_epi_grav **epi, const int *n_epi, const int **id_epj,
                            const int *n_epj, const int **id_spj, const int *n_spj, const sph_epj_grav *epj,
                            int n_epj_tot, const sph_spj_monopole *spj, int n_spj_tot, int send_flag);
/* message of the last failed batch call on this thread */
const char *sph_batch_last_error(void);
/* Arithmetic of the dispatches that follow (all tags): SPH_PREC_FP64 (default) runs the reference
 * functors in FP64; SPH_PREC_MIXED runs the same walks with the pair terms in FP32 on coordinates
 * and velocities relative to each walk's first i-particle (double-float), compensated FP32 sums and
 * FP64 per-particle epilogues -- the device-resident mixed path's arithmetic, within 1e-5 of FP64
 * on the functors' results.  No counterpart in the reference (its functors are FP64). */
int sph_batch_set_precision(int precision);
/* Who moves a dispatch's walks to the device (all tags).  SPH_BATCH_STAGING_AUTO (default): the GPU
 * reads them from the caller's arrays with a gather kernel where it can read pageable host memory
 * (cudaDevAttrPageableMemoryAccess; GB300's NVLink-C2C) and every array is 8-byte aligned, else
 * the host copies them into pinned staging.  _HOST: always the host copy.  _DEVICE: always the
 * gather; a dispatch that cannot gather fails with SPH_ERR_STATE.  Either way a dispatch returns
 * after it has read the caller's arrays, so they may be reused at once.  No counterpart in the
 * reference. */
#define SPH_BATCH_STAGING_AUTO 0
#define SPH_BATCH_STAGING_HOST 1
#define SPH_BATCH_STAGING_DEVICE 2
int sph_batch_set_staging(int mode);

/* ---- 2. device-resident whole-pass API ----------------------------------- */

/* Field-major particle block: field f of particle i is at fields[f * ld + i]
 * (ld >= n).  Field order: */
enum sph_field {
    SPH_X = 0, SPH_Y, SPH_Z, SPH_VX, SPH_VY, SPH_VZ, SPH_MASS, SPH_SMTH, SPH_DENS, SPH_ENG,
    SPH_PRES, SPH_SNDS, SPH_DIVV, SPH_ROTX, SPH_ROTY, SPH_ROTZ, SPH_BAL, SPH_AVA, SPH_GRADH,
    SPH_AX, SPH_AY, SPH_AZ, SPH_ENGDOT, SPH_VHX, SPH_VHY, SPH_VHZ, SPH_ENGHALF, SPH_DT,
    SPH_GX, SPH_GY, SPH_GZ, SPH_POT,
    SPH_ENT, SPH_TEMP,       /* entropy and temperature (class.h:96-98), written by mode 2 */
    SPH_NFIELD
};

#define SPH_PREC_FP64 0    /* every pair sum in FP64 (parity path) */
#define SPH_PREC_MIXED 1   /* FP32 pair sums on group-relative coordinates, FP64 everywhere else */

typedef struct {
    double theta;            /* gravity opening angle (0.5, main.cpp:90) */
    int32_t n_leaf;          /* octree leaf limit (8, main.cpp:90) */
    int32_t n_group;         /* gravity i-group limit (256, main.cpp:90) */
    int32_t n_dens_iter;     /* density passes per step (4: param.h:11, main.cpp:138) */
    int32_t self_gravity;    /* 1 = SELF_GRAVITY (GI.h:4) */
    int32_t ext_damp;        /* 1 = GI_universal::addExternalForce (GI.h:458-465) */
    int32_t precision;       /* SPH_PREC_FP64 or SPH_PREC_MIXED */
    double ext_damp_tend;    /* 5000 s in the reference */
    double damping;          /* dampMotion factor (1.0) */
    double G;                /* 6.67e-11 (force.h:171-172) */
    int32_t device;          /* CUDA device ordinal */
    int32_t mode;            /* 1 or 2 ("mode", main.cpp:115): 2 ends every step with
                                SetConstantEntropy + CalcAll (main.cpp:155-158, force.h:55-84) */
    double mantle_entropy;   /* entropy of material 0 in mode 2 ("mantle_entropy", main.cpp:116-117) */
    double core_entropy;     /* entropy of every other material ("core_entropy", main.cpp:118-119) */
    int32_t entropy_grid;    /* grid_length of RestrictedBilinearInterpolation: 120, the constant
                                EoS.h:250-251 and 403-404 pass */
    int32_t entropy_abs;     /* distance in its nearest-entropy search (interpolation.h:199-200):
                                SPH_ENTROPY_ABS_INT (the reference compiled with main.cpp's own
                                includes: unqualified abs() of a double resolves to int abs(int),
                                so distances are truncated to integers) or SPH_ENTROPY_ABS_REAL */
} sph_config;

#define SPH_ENTROPY_ABS_INT 0
#define SPH_ENTROPY_ABS_REAL 1

typedef struct sph_ctx sph_ctx;

void sph_config_default(sph_config *cfg);
int sph_ctx_create(const sph_config *cfg, sph_ctx **out);
int sph_ctx_destroy(sph_ctx *ctx);
const char *sph_last_error(const sph_ctx *ctx);

/* EoS materials, indexed by the per-particle material id.
 * Table mode mirrors BilinearInterpolation (interpolation.h:33-102) on the
 * reference's rho-u tables (EoS.h:121-221): rho axis [n_rho], u axis [n_u],
 * pressure and sound-speed planes [n_rho * n_u] rho-major. */
int sph_set_eos_table(sph_ctx *ctx, int material, const double *rho_axis, int n_rho, const double *u_axis,
                      int n_u, const double *pres, const double *snds);
/* Reads a rho-u text table (EoS.h:121-221 format) into material slot `material`. */
int sph_load_eos_table_file(sph_ctx *ctx, int material, const char *path);
/* The same reader into host arrays, with no context and no device work (the reference's table
 * constructor, EoS.h:121-221, reads the file the same way).  Pass null arrays first to get
 * *n_rho, *n_u and *n_cols (6, or 5 for a file without the entropy column); then rho[n_rho]
 * (column 0 of each density block's first line), u[n_u] (column 1 of the first block's lines)
 * and cols[6 * n_rho * n_u], column c of file line l at cols[c * n_rho * n_u + l] (the entropy
 * column zero when absent).  SPH_ERR_TABLE for a missing or malformed file;
 * sph_read_eos_table_error() gives the message (per thread). */
int sph_read_eos_table_file(const char *path, int *n_rho, int *n_u, double *rho, double *u, double *cols,
                            int *n_cols);
const char *sph_read_eos_table_error(void);
/* Analytic Tillotson: rho0 u0 uiv ucv A B a b alpha beta (EoS.h:116-238 parameter order). */
int sph_set_eos_tillotson(sph_ctx *ctx, int material, const double par[10]);
/* Ideal gas (EoS.h:37-66) with heat-capacity ratio gamma. */
int sph_set_eos_ideal(sph_ctx *ctx, int material, double gamma);
/* The columns of a table material that mode 2 reads (call after
 * sph_set_eos_table for the same slot; sph_load_eos_table_file sets them):
 * temperature (column 2) and entropy (column 5) planes [n_rho * n_u], and the
 * density and energy columns of every table line, line_rho / line_u
 * [n_rho * n_u] (columns 0 and 1 in file order; the reference's
 * full_densities / full_energies, EoS.h:290-390; NULL = the axes repeated).
 * line_rho must be non-decreasing. */
int sph_set_eos_entropy(sph_ctx *ctx, int material, const double *temp, const double *ent,
                        const double *line_rho, const double *line_u);

/* The EoS surface of EoS_t (EoS.h:11-31) on the device, for n points in host
 * memory: out[i] = quantity(a[i], b[i]) of `material`.  Quantities:
 *   SPH_EOS_PRESSURE, SPH_EOS_SOUND_SPEED   (rho, u)  EoS.h:241-247, 394-400
 *   SPH_EOS_TEMPERATURE, SPH_EOS_ENTROPY    (rho, u)  EoS.h:254-260, 407-413
 *   SPH_EOS_INTERNAL_ENERGY                 (rho, s)  EoS.h:249-252, 402-405
 * (ideal gas: EoS.h:43-61).  INTERNAL_ENERGY uses the context's entropy_grid
 * and entropy_abs; a lookup whose reference evaluation would index outside
 * its vectors (undefined there) returns NaN and is counted in *undefined
 * (may be null). */
#define SPH_EOS_PRESSURE 0
#define SPH_EOS_SOUND_SPEED 1
#define SPH_EOS_TEMPERATURE 2
#define SPH_EOS_ENTROPY 3
#define SPH_EOS_INTERNAL_ENERGY 4
int sph_eos_eval(sph_ctx *ctx, int material, int quantity, int64_t n, const double *a, const double *b,
                 double *out, int64_t *undefined);

/* Copies n particles (host memory) into the context; particle i keeps slot i
 * for download.  flags:
 *   SPH_UPLOAD_INIT_SMTH    apply RealPtcl::initialize (class.h:196-199:
 *                           h = 1.2 (m / rho)^(1/3), grad_smth = 1);
 *   SPH_UPLOAD_FORCES_VALID the block's acc / grav / eng_dot / dt fields are
 *                           the forces of this state and `dt` is the global
 *                           step (system_t::dt, class.h:9), so sph_step may
 *                           run without a prologue: a host that keeps its
 *                           particles (as the reference's ParticleSystem does)
 *                           can upload, step and download every step;
 *   SPH_UPLOAD_STEP_INPUTS  copy only the fields a step reads or carries
 *                           unchanged (SPH_STEP_INPUT_FIELDS: positions,
 *                           velocities, mass, smth, eng, AVa, acc, eng_dot,
 *                           grav, ent, temp); the rest are outputs of the next
 *                           step and read as zero until it has run.
 * Masses must be positive and finite and every material set (checked on the
 * device; SPH_ERR_NONFINITE / SPH_ERR_ARG). */
#define SPH_UPLOAD_INIT_SMTH 1
#define SPH_UPLOAD_FORCES_VALID 2
#define SPH_UPLOAD_STEP_INPUTS 4
#define SPH_FIELD_BIT(f) (1ull << (f))
#define SPH_STEP_INPUT_FIELDS                                                                                     \
    (SPH_FIELD_BIT(SPH_X) | SPH_FIELD_BIT(SPH_Y) | SPH_FIELD_BIT(SPH_Z) | SPH_FIELD_BIT(SPH_VX) |                \
     SPH_FIELD_BIT(SPH_VY) | SPH_FIELD_BIT(SPH_VZ) | SPH_FIELD_BIT(SPH_MASS) | SPH_FIELD_BIT(SPH_SMTH) |         \
     SPH_FIELD_BIT(SPH_ENG) | SPH_FIELD_BIT(SPH_AVA) | SPH_FIELD_BIT(SPH_AX) | SPH_FIELD_BIT(SPH_AY) |           \
     SPH_FIELD_BIT(SPH_AZ) | SPH_FIELD_BIT(SPH_ENGDOT) | SPH_FIELD_BIT(SPH_GX) | SPH_FIELD_BIT(SPH_GY) |        \
     SPH_FIELD_BIT(SPH_GZ) | SPH_FIELD_BIT(SPH_ENT) | SPH_FIELD_BIT(SPH_TEMP))
int sph_upload(sph_ctx *ctx, int64_t n, const double *fields, int64_t ld, const int64_t *id,
               const int32_t *material, double time, double dt, int flags);
/* Copies the state back in upload order. */
int sph_download(sph_ctx *ctx, double *fields, int64_t ld, int64_t *id, int32_t *material);
/* The same for the fields in field_mask only (bit f = field f; the other rows of `fields` are
 * left as they are; id / material may be NULL).  A host that keeps its particles can read back
 * SPH_STEP_OUTPUT_FIELDS after each step: every field a step writes. */
int sph_download_fields(sph_ctx *ctx, double *fields, int64_t ld, uint64_t field_mask, int64_t *id,
                        int32_t *material);
#define SPH_STEP_OUTPUT_FIELDS (~(SPH_FIELD_BIT(SPH_MASS) | SPH_FIELD_BIT(SPH_AVA) | SPH_FIELD_BIT(SPH_ENT) | \
                                  SPH_FIELD_BIT(SPH_TEMP)) & (SPH_FIELD_BIT(SPH_NFIELD) - 1))
#define SPH_STEP_OUTPUT_FIELDS_MODE2 (SPH_STEP_OUTPUT_FIELDS | SPH_FIELD_BIT(SPH_ENT) | SPH_FIELD_BIT(SPH_TEMP))
/* Forces of the current state and the first dt (main.cpp:92-105). */
int sph_prologue(sph_ctx *ctx);
/* n_steps iterations of the loop body of main.cpp:125-173.  In mode 2 each
 * step ends, after the final kick, with ent = mantle_entropy for material 0
 * and core_entropy otherwise (SetConstantEntropy, force.h:55-65), then
 * eng = InternalEnergy(dens, ent) and temp = Temperature(dens, eng) (CalcAll,
 * force.h:73-84); a lookup that is undefined in the reference or gives a
 * non-finite energy fails the step with SPH_ERR_NONFINITE. */
int sph_step(sph_ctx *ctx, int n_steps);
/* One sph_step that also copies the fields in field_mask (e.g. SPH_STEP_OUTPUT_FIELDS) into the
 * host block `fields` (field-major, leading dimension ld, upload order), each as soon as the
 * step has finished writing it, so the copies overlap the rest of the step (host memory should
 * be pinned for that).  The other rows of `fields` are left as they are. */
int sph_step_download(sph_ctx *ctx, double *fields, int64_t ld, uint64_t field_mask);
int sph_get_time(const sph_ctx *ctx, double *time, double *dt, int64_t *step);

/* Conserved quantities in FP64: E = sum m (u + v^2/2 + pot/2), P = sum m v,
 * L = sum m x cross v.  out[0] = E, out[1..3] = P, out[4..6] = L, out[7] = sum m.
 * Summed over the context's runs. */
int sph_diagnostics(sph_ctx *ctx, double out[8]);

/* ---- several runs in one context (batching and serving) -------------------
 * No counterpart in the reference, which advances one ParticleSystem per
 * process (main.cpp:69-173).  A context holds any number of independent runs
 * (impacts of their own size); each has its own root cube, octree, time and
 * global dt (getTimeStepGlobal per run, integral.h:4-20), and one set of
 * launches per pass advances all of them.  sph_upload makes a context with one
 * run; sph_add_run appends a run (its handle is returned) and may be called
 * between steps; a run added without valid forces takes its first sph_step as
 * its prologue (main.cpp:92-105: forces and dt, no kick).  sph_remove_run
 * drops a run's particles; sph_download_run copies one run back in its upload
 * order.  Results of a run do not depend on the other runs in the context.
 * sph_add_run returns SPH_ERR_ARG for a run whose mean particle mass differs
 * from the run set's first run by more than a factor 2^60 (the FP32 mass
 * copies share the first run's scale). */
int sph_add_run(sph_ctx *ctx, int64_t n, const double *fields, int64_t ld, const int64_t *id,
                const int32_t *material, double time, double dt, int flags, int64_t *handle);
int sph_remove_run(sph_ctx *ctx, int64_t handle);
int sph_list_runs(sph_ctx *ctx, int64_t *handles, int cap, int *n_runs);
int sph_run_info(sph_ctx *ctx, int64_t handle, int64_t *n, double *time, double *dt, int64_t *steps);
int sph_download_run(sph_ctx *ctx, int64_t handle, double *fields, int64_t ld, int64_t *id, int32_t *material);
int sph_run_diagnostics(sph_ctx *ctx, int64_t handle, double out[8]);

/* ---- launch-shape autotuner (mixed precision) ------------------------------
 * No counterpart in the reference.  mode 0: times the derivative and hydro
 * kernels with 1, 2 and 4 threads per i-particle on the context's current
 * state and lists (call after sph_step; the state is left unchanged), keeps
 * the fastest and returns params[0] = derivative, params[1] = hydro threads
 * per particle, params[2..4] / [5..7] = the measured times in microseconds.
 * mode 1: applies params[0], params[1].  The choice changes the summation
 * order of the FP32 pair sums only (rounding level). */
int sph_autotune(sph_ctx *ctx, int mode, int64_t params[8]);

/* ---- inspection (tests, tooling) ----------------------------------------- */
/* Runs only the given pass on the current state (positions unchanged):
 * 0 = sort + tree, 1 = one density pass, 2 = EoS, 3 = derivative, 4 = hydro, 5 = gravity. */
int sph_run_pass(sph_ctx *ctx, int pass);
/* Current particle order (sorted): slot of the k-th particle, Morton keys. */
int sph_get_order(sph_ctx *ctx, int32_t *slot, uint64_t *keys);
/* SPH neighbour list of the k-th particle in sorted order for the last built
 * list of the given mode (0 gather, 1 symmetric); writes ascending sorted
 * indices, returns the count in *n (may exceed cap). */
int sph_get_neighbors(sph_ctx *ctx, int mode, int64_t k, int32_t *out, int64_t cap, int64_t *n);
/* Octree summary: number of cells and, per cell, start/count/level/n_child (arrays may be null). */
int sph_get_tree(sph_ctx *ctx, int64_t *n_cell, int32_t *start, int32_t *count, int32_t *level, int32_t *n_child,
                 double *com_mass /* [4 * n_cell] x y z m */);
/* Gravity interaction list of group g: EPJ sorted indices and SPJ cells as (level, start). */
int sph_get_grav_list(sph_ctx *ctx, int64_t g, int64_t *n_group, int32_t *epj, int64_t cap_epj, int64_t *n_epj,
                      int32_t *spj_level, int32_t *spj_start, int64_t cap_spj, int64_t *n_spj,
                      int32_t *group_start, int32_t *group_count);
/* Every gravity interaction list of the last FP64 gravity pass in a few copies (tooling: a host
 * that builds calcForceAllAndWriteBackMultiWalk walks from the device's tree).  Per group g: its
 * first sorted particle and count, and the offset and length of its EPJ run (sorted particle
 * indices in epj) and SPJ run (cell indices into sph_get_tree's arrays in spj_cell).  Null arrays
 * are skipped; *n_group, *n_epj_total and *n_spj_total are always written. */
int sph_get_grav_lists(sph_ctx *ctx, int64_t *n_group, int64_t *n_epj_total, int64_t *n_spj_total,
                       int32_t *group_start, int32_t *group_count, int32_t *epj_off, int32_t *epj_len, int32_t *epj,
                       int32_t *spj_off, int32_t *spj_len, int32_t *spj_cell);
/* Device time (CUDA events on the context's stream) accumulated per segment
 * since the last reset, in this order: kick-drift-predict, octree levels and
 * moments, density lists, density kernels, EoS, derivative list, derivative
 * kernel, hydro list, hydro kernel, gravity groups (and lists on the FP64
 * path), gravity kernel, final kick + dt, key sort + permutation, neighbour
 * walk preparation, mode-2 entropy step (SetConstantEntropy + CalcAll).
 * cap = -1 switches timing on (and resets), -2 switches it off, -3 resets. */
int sph_get_timings(sph_ctx *ctx, double *ms, int cap, int *n);
/* sph_step bracketed by CUDA events on the context's stream; device_ms = elapsed. */
int sph_step_timed(sph_ctx *ctx, int n_steps, double *device_ms);
/* out[0] kernels launched by the context so far; out[1] gather-list pairs (one
 * density / derivative pass); out[2] symmetric-list pairs (hydro); out[3]
 * gravity interactions (sum over groups of n_i x (EPJ + SPJ)); out[4] cells;
 * out[5] gravity groups; out[6] EPJ entries; out[7] SPJ entries; out[8]
 * full neighbour-superset walks; out[9] partial (repair) walks; out[10]
 * particles whose h outgrew the superset skin; out[11] walk units walked;
 * out[12] walk units; out[13] superset row capacity; out[14] superset entries;
 * out[15] superset entries in spill ranges (rows longer than the capacity). */
int sph_get_counters(sph_ctx *ctx, int64_t out[16]);
/* ---- allocation-free Morton ordering -------------------------------------
 * No counterpart in the reference: FDPS builds its tree on the host.  This
 * is the key-and-sort stage of the device octree build for callers that
 * must not allocate device memory: a host that runs under a fixed
 * device-memory budget (its own pool allocator owns the rest of the GPU),
 * or one that may not take the device-wide synchronisation of a cudaFree in
 * the middle of its step.  The call returns after its work on `stream` has
 * finished when called eagerly (it reads a status word back).  x, y, z
 * (n doubles each), keys_out (n) and order_out (n) are device pointers;
 * stream may be null (the legacy default stream).  keys_out[k] is the k-th
 * smallest 63-bit Morton key over the octree's root cube and order_out[k]
 * the index of that particle (stable: ties keep input order), bit-identical
 * to the order sph_run_pass(ctx, 0) produces for the same positions.
 * Scratch lives in one file-scope device array for at most
 * SPH_NOALLOC_MAX_N particles (about 3.2 MB, present on every GPU that loads
 * the library); larger n returns SPH_ERR_CAPACITY, null pointers or n < 1
 * SPH_ERR_ARG, a non-finite position SPH_ERR_NONFINITE, a CUDA error already
 * pending on the calling thread SPH_ERR_CUDA (before any work is queued; the
 * error is left in place).  The first call on a
 * device looks up the array's device address (cudaGetSymbolAddress) and must
 * not be made while `stream` is being captured (SPH_ERR_STATE, nothing
 * recorded).  Called eagerly, the call ends by reading its error word back
 * and synchronising `stream`, so it returns after its work is done.  Called
 * while `stream` is being captured into a CUDA graph, it records its work
 * (a memset, kernel launches, device-to-device copies) and returns SPH_OK at
 * once; a replay of the graph reports no status (a non-finite position then
 * leaves its key undefined).  Every call on a device shares the array: calls
 * (or replays) that overlap on the GPU race.  No device memory is allocated
 * or freed. */
#define SPH_NOALLOC_MAX_N 131072
int sph_morton_order_noalloc(const double *x, const double *y, const double *z, int64_t n, uint64_t *keys_out,
                             int32_t *order_out, void *stream);

/* Measures the FP32 (fp64 = 0) or FP64 (fp64 = 1) fused-multiply-add rate of
 * the device in TFLOP/s (2 flops per FMA): the roofline of the pair kernels. */
int sph_probe_peak(int device, int fp64, double *tflops);

#ifdef __cplusplus
}
#endif
#endif
