// Internal declarations shared by the translation units of libsph_gb300.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <string>
#include <vector>

#include "../../include/sph_gb300.h"

namespace sph {

constexpr int KEY_LEVELS = 21;           // 3 x 21-bit Morton key
constexpr int MAX_LEVELS = KEY_LEVELS + 1;
constexpr int MAX_MATERIALS = 16;
constexpr double SUPPORT = 2.5;          // kernel.h:36-38
constexpr double SMTH_COEF = 1.2;        // param.h:9
constexpr double C_CFL = 0.3;            // param.h:10
constexpr double AV_STRENGTH = 1.0;      // param.h:17
constexpr double DENS_FLOOR = 5.0;       // force.h:18-20 (FLAG_GI)

// device-side error word bits
constexpr int ERR_SPH_LIST_OVERFLOW = 1;
constexpr int ERR_CELL_OVERFLOW = 2;
constexpr int ERR_GRAV_OVERFLOW = 4;
constexpr int ERR_NONFINITE = 8;
constexpr int ERR_SPH_STACK = 32;         // SPH walk stack overflow

// Double-float accumulation in FP32 (Knuth's TwoSum): hi + lo carries a
// running sum to about 2^-44 relative without touching the FP64 pipe, which
// on this GPU issues at a small fraction of the FP32 rate.
__device__ __forceinline__ void df_add(float &hi, float &lo, float a) {
    const float s = __fadd_rn(hi, a);
    const float bp = __fsub_rn(s, hi);
    const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bp)), __fsub_rn(a, bp));
    hi = s;
    lo = __fadd_rn(lo, e);
}

// Hardware approximations for the FP32 pair arithmetic of the mixed kernels
// (relative error about 2^-22, denormals flushed): one MUFU instruction each
// instead of the IEEE-rounded sequences that sqrtf and '/' compile to.
__device__ __forceinline__ float rsqrt_a(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp_a(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float sqrt_a(float x) {
    float y;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// packed pairs of FP32 values in one 64-bit register (low half first) and the paired FP32
// arithmetic of sm_100+ (one instruction, two IEEE round-to-nearest results)
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 f2_pack(float a, float b) {
    f32x2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void f2_unpack(f32x2 r, float &a, float &b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ f32x2 f2_add(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 f2_sub(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 f2_mul(f32x2 a, f32x2 b) {
    f32x2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f32x2 f2_fma(f32x2 a, f32x2 b, f32x2 c) {
    f32x2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

// Neighbour rows: particle i's first K entries at i * K; the rare particles
// with more (isolated particles whose h grew towards the body's size have
// thousands) continue in a spill range of the same allocation, entries K..
// at main + soff[i] (main = the row block's size; soff: exclusive prefix of the
// spill lengths, n + 1 entries, multiples of 8).  soff == nullptr: no spill.
struct RowMap {
    int K = 0;
    int64_t main = 0;
    const int *soff = nullptr;
};

// start of segment `seg` (0 = the row, 1 = its spill) of particle i's c entries, and its length
__device__ __forceinline__ int64_t row_seg(const RowMap &m, int64_t i, int seg, int c, int *len) {
    if (seg == 0) {
        *len = c < m.K ? c : m.K;
        return i * m.K;
    }
    *len = c - m.K;
    return (*len > 0 && m.soff) ? m.main + m.soff[i] : 0;
}

// particle i's row over its logical positions 0 .. c - 1: positions below K sit in the row
// block, the others in the spill range.  Kernels that split a row between threads or flush
// partial sums every so many entries count positions on this view, so how the entries group
// does not depend on K (which follows the row lengths of every run in the context).  K is a
// multiple of 8, so an aligned pair or quad of positions never straddles the two parts.
struct RowView {
    const int *blk, *spill;   // spill is offset by -K: spill[k] for k >= K
    int K, c;
    __device__ __forceinline__ const int *at(int k) const { return (k < K ? blk : spill) + k; }
};

__device__ __forceinline__ RowView row_view(const int *nbr, const RowMap &m, int64_t i, int c) {
    RowView v;
    v.K = m.K;
    v.blk = nbr + i * m.K;
    const bool sp = c > m.K && m.soff;
    v.spill = sp ? nbr + m.main + m.soff[i] - m.K : v.blk;
    v.c = (c > m.K && !sp) ? m.K : c;
    return v;
}

__device__ __forceinline__ int row_spill_cap(const RowMap &m, int64_t i) {
    return m.soff ? m.soff[i + 1] - m.soff[i] : 0;
}

// Mixed-precision tail of a density pass (force.h:32-41): rho = max(floor,
// sum_j m_j w_j x norm) and h = 1.2 (m / rho)^(1/3), in FP32.  dscale =
// (1365/64) / (pi mscale) carries the kernel constant and the mass scale;
// invH = 1 / (2.5 h).
__device__ __forceinline__ void density_tail32(float sum, float invH, float dscale, double m, double *rho,
                                               double *h) {
    const float d = fmaxf((float)DENS_FLOOR, sum * dscale * (invH * invH * invH));
    *rho = (double)d;
    *h = (double)((float)SMTH_COEF * cbrtf((float)m / d));
}

// One slice of RestrictedBilinearInterpolation (interpolation.h:131-238) for a
// fixed entropy: the slice's first line density and the energy interpolated
// at that entropy between the slice's two entries nearest to it.
struct EntropyEdge {
    double p, u;
    int undef, pad;      // undef: the reference indexes outside its vectors here
};

struct DevMaterial {
    int kind;            // 0 table, 1 Tillotson, 2 ideal gas, -1 unset
    int n_rho, n_u, pad;
    const double *rho, *u, *pres, *snds;
    double par[10];
    // mode-2 columns of a table (null: none): temperature and entropy planes,
    // density and energy of every line (file order)
    const double *temp, *ent, *line_rho, *line_u;
    // mode-2 slices at the material's entropy: lower by (last line <= rho) + 1,
    // upper by (first line >= rho), n_rho * n_u + 1 entries each
    const EntropyEdge *edge_lo, *edge_up;
};

// tree meta block (ints): level l cells are [meta[l], meta[l+1]) for l = 0..21;
// meta[MAX_LEVELS] = total cells, META_ERR = error bits.
constexpr int META_N = 64;
constexpr int META_ERR = 40;
constexpr int META_NGROUP = 41;
constexpr int META_MAXCNT = 42;   // max SPH neighbour count seen by the last list build
constexpr int META_NEPJ = 43;     // total gravity EPJ entries
constexpr int META_NSPJ = 44;     // total gravity SPJ entries

struct Tree {
    int64_t cap = 0;
    int *start = nullptr, *count = nullptr, *level = nullptr, *first_child = nullptr, *n_child = nullptr,
        *parent = nullptr;
    double4 *mom = nullptr;   // (m x, m y, m z, m)
    double4 *com = nullptr;   // (com x, y, z, m)
    float4 *blo = nullptr;    // bbox lower corner (rounded down), .w unused
    float4 *bhi = nullptr;    // bbox upper corner (rounded up), .w = hmax (rounded up)
    int *tmp_cnt = nullptr, *tmp_off = nullptr, *tmp_b = nullptr;
    int4 *cinfo = nullptr;    // per cell: first_child, n_child, start, count
    int *meta = nullptr;      // device [META_N]
    double *rb = nullptr;     // device, per run (stride RB_STRIDE): root_lo[3], root_len, scale, rc2[MAX_LEVELS] at [8..]
    int rb_cap = 0;           // runs rb has room for
    int n_cell_host = 0;
    int depth = KEY_LEVELS;   // the last tree's deepest level
};

struct Sort {
    int64_t cap = 0;
    uint64_t *k0 = nullptr, *k1 = nullptr;
    uint32_t *v0 = nullptr, *v1 = nullptr;
    uint32_t *hist = nullptr;   // [256 * nblocks]
    uint32_t *hoff = nullptr;
    int nblocks_cap = 0;
};

struct SphLists {
    int64_t pitch = 0;   // row stride: particle i's neighbours at nbr[i * pitch + k], k < cnt[i]
    int K = 0;           // capacity per particle
    int K_alloc = 0;     // allocated capacity per particle
    int *nbr = nullptr;  // [n * K]
    int *cnt = nullptr;  // [n]
    bool valid = false;
};

struct GravLists {
    int64_t cap_groups = 0, cap_epj = 0, cap_spj = 0;
    int *group_cell = nullptr;   // [ng]
    int *is_group = nullptr;     // [cell cap] scratch
    int *n_epj = nullptr, *n_spj = nullptr;          // [ng]
    int *off_epj = nullptr, *off_spj = nullptr;      // [ng]
    int *epj = nullptr, *spj = nullptr;
    int ng = 0;
    int64_t tot_epj = 0, tot_spj = 0;
    bool valid = false;          // epj / spj lists filled
    bool counts_valid = false;   // n_epj / n_spj filled (by the lists or by the fused walk)
};

// per-step SPH neighbour superset (sph_nbr.cu)
struct SphSuper {
    int64_t pitch = 0, cap_particles = 0, cap_units = 0;
    int K = 0, K_alloc = 0;
    int *nbr = nullptr, *cnt = nullptr;   // superset, ELL
    float *r2 = nullptr;                  // FP32 r^2 of every superset entry
    float *m = nullptr;                   // neighbour mass x mscale of every superset entry
    double *hsup = nullptr;               // h when the superset was built
    float4 *pxh = nullptr, *pxl = nullptr;  // double-float positions
    float *H2f = nullptr;                 // (2.5 h)^2 rounded up
    int2 *units = nullptr;                // (start, count) of the walk units
    int n_units = 0;
    bool valid = false;
    int64_t rebuilds = 0;    // full walks
    int64_t repairs = 0;     // partial walks after h outgrew the skin
    int64_t violators = 0;   // particles that outgrew the skin
    int64_t units_walked = 0;
    int rebuilds_step = 0;   // superset walks since the last sort
    // repair scratch
    float *vR = nullptr, *cvR = nullptr;
    int *umark = nullptr, *uoff = nullptr, *uidx = nullptr;
    int64_t cap_cells = 0;
    // spill of the rows longer than K (RowMap): offsets, their capacity, units holding such rows
    int64_t main = 0;             // K * rows: where the spill ranges start in nbr / r2 / m / the lists
    int64_t spill_cap = 0;        // entries each array holds beyond `main`
    int *soff = nullptr;          // [n + 1]
    int *need = nullptr;          // [n + 1] scratch
    int *uover = nullptr;         // per unit: some row of the unit is longer than K
    int *npass = nullptr;         // [pitch] density passes a particle has completed this step
    bool spill_on = false;        // soff holds this sort's spill layout
    int64_t spill_alloc = 0;      // spill_cap the arrays were allocated with
    int64_t cap_soff = 0, cap_uover = 0;
    int64_t spilled = 0;          // entries spilled at the last layout (counter)
    RowMap map() const {
        RowMap r;
        r.K = K;
        r.main = main;
        r.soff = spill_on ? soff : nullptr;
        return r;
    }
};

struct Scan {
    int *part = nullptr;   // [SCAN_BLOCKS + 1]
    int *total = nullptr;  // device int
};

// Runs: independent simulations advanced together by one context (one set of
// launches per pass for all of them).  A run's particles are contiguous, runs
// in index order, each in its own key order; every run has its own root cube,
// octree root (cell r of level 0), dt and time.  sph_upload makes one run.
constexpr int RUN_TILE = 2048;    // sort / reduction tile, aligned to run starts
constexpr int RB_STRIDE = 32;     // doubles per run in Tree::rb
struct Runs {
    int R = 0;
    std::vector<int64_t> n, off;            // particles per run, first particle
    std::vector<double> time, dt;           // host copies; dt of the coming step
    std::vector<int64_t> steps, handle;
    std::vector<int> fresh;                 // joined since the last step: its first step is its prologue
    std::vector<int> mexp;                  // the run's own mass scale 2^mexp (~ 1 / its mean mass)
    std::vector<double> mmax;               // the run's largest particle mass
    bool fix_split = true;                  // every run's largest mass x its own scale <= 15
    int T = 0;                              // tiles over all runs
    int cap_R = 0, cap_T = 0;
    int4 *tiles = nullptr;                  // device [T]: start, length, histogram base, tiles of its run
    int4 *info = nullptr;                   // device [R]: first particle, particles, first tile, tiles
    double *dt_dev = nullptr;               // device [R]: dt of the coming step
    double *part = nullptr;                 // device [T * 8]: per-tile partials
    double *out = nullptr;                  // device [R * 8]: per-run results
    unsigned char *damp = nullptr;          // device [R]: external damping applies
    int *fixd = nullptr;                    // device [R]: log2 of the context's mass scale over the run's
    int *prun = nullptr, *prun2 = nullptr;  // device [cap]: run of each particle (permuted with it)
    int64_t next_handle = 1;
};

}  // namespace sph

namespace sph {
constexpr int GRAPH_KEY_N = 21;
// a captured sort + octree build and what it was captured for
struct TreeGraph {
    cudaGraphExec_t exec = nullptr;
    uintptr_t key[GRAPH_KEY_N] = {0};
    int64_t launches = 0;
};
}  // namespace sph

struct sph_ctx {
    sph_config cfg;
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    // sph_step_download: fields go to the host on their own stream as soon as the step has
    // finished writing them (unpermuted into dl_buf first)
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t dl_ev[8] = {nullptr};
    int dl_next = 0;
    double *dl_buf = nullptr;      // [SPH_NFIELD][cap], upload order
    int64_t dl_cap = 0;
    double *dl_host = nullptr;     // the request: host block, its leading dimension, fields left
    int64_t dl_ld = 0;
    uint64_t dl_left = 0;
    std::string err;

    int64_t n = 0, cap = 0;
    double *F = nullptr, *F2 = nullptr;     // [SPH_NFIELD][cap] master state in sorted order
    int64_t *id = nullptr, *id2 = nullptr;
    int32_t *slot = nullptr, *slot2 = nullptr;
    int32_t *mat = nullptr, *mat2 = nullptr;
    uint64_t *keys = nullptr;               // sorted keys of the current order
    double *scratch_d = nullptr;            // reductions [64]
    double *host_scalars = nullptr;         // pinned [64]

    // mixed-precision packed copies (double-float hi/lo)
    float4 *xh = nullptr, *xl = nullptr, *vhf = nullptr, *vlf = nullptr;

    sph::DevMaterial mats_host[sph::MAX_MATERIALS];
    std::vector<void *> table_allocs;
    sph::DevMaterial *mats_dev = nullptr;

    sph::Tree tree;
    sph::Sort sort;
    sph::SphLists lists[2];
    sph::SphSuper sup;
    sph::GravLists grav;
    sph::Scan scan;
    sph::Runs runs;

    double mscale = 1.0;   // power of two ~ 1 / particle mass, keeps FP32 pair sums near unity
    int mexp = 0;          // mscale = 2^mexp, set by the first run of a run set

    int64_t step = 0;          // steps taken by sph_step (all runs)
    bool uploaded = false;
    bool have_forces = false;   // sph_upload contexts: the prologue (or the uploaded forces) came first
    bool batch = false;         // runs added with sph_add_run: a new run's first step is its prologue

    // per-segment device timings (CUDA events on `stream`), accumulated until reset
    cudaEvent_t ev[64];
    int mark_seg[64];
    int n_ev = 0;
    double seg_ms[16] = {0};
    int64_t seg_calls[16] = {0};
    bool timing = false;
    cudaEvent_t ev_begin = nullptr, ev_end = nullptr;

    int64_t launches = 0;   // kernels launched by this context

    // launch shapes of the mixed kernels (sph_autotune); the defaults are the untuned choice
    struct {
        int drvt_tpi = 1, hydro_tpi = 1;   // threads per i-particle
    } tune;

    // mode 2 (SetConstantEntropy + CalcAll, sph_entropy.cu)
    int *m2_bad = nullptr;                             // device: failed lookups of the last entropy step
    bool m2_dirty = true;                              // materials changed since the slices were built
    void *m2_edges[sph::MAX_MATERIALS] = {nullptr};    // per material: edge_lo and edge_up

    // CUDA graphs of the sort + octree build: one per state-buffer parity and layout
    bool use_graphs = true;
    sph::TreeGraph tree_graphs[4];
    int graph_next = 0;
    int64_t graph_captures = 0, graph_replays = 0;
};

// timing segments, in the order sph_get_timings reports them
enum {
    SEG_KDP = 0, SEG_TREE, SEG_DENS_LIST, SEG_DENS, SEG_EOS, SEG_DRVT_LIST, SEG_DRVT, SEG_HYDRO_LIST, SEG_HYDRO,
    SEG_GRAV_LIST, SEG_GRAV, SEG_FINAL,
    SEG_SORT,       // root box, keys, radix sort, permutation (before SEG_TREE: levels and moments)
    SEG_NBR_PREP,   // walk units, cell reach, mixed-precision packs (after SEG_TREE)
    SEG_ENTROPY,    // mode 2: SetConstantEntropy + CalcAll
    SEG_N
};

// ---------------------------------------------------------------------------
// host helpers (sph_api.cu)
int sph_fail(sph_ctx *ctx, int code, const char *fmt, ...);
#define SPH_CUDA(ctx, call)                                                                                 \
    do {                                                                                                    \
        cudaError_t e_ = (call);                                                                            \
        if (e_ != cudaSuccess) return sph_fail((ctx), SPH_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call, \
                                               cudaGetErrorString(e_));                                    \
    } while (0)
#define SPH_TRY(x)                \
    do {                          \
        int rc_ = (x);            \
        if (rc_ != SPH_OK) return rc_; \
    } while (0)

// tree / sort (sph_tree.cu)
int sph_tree_reserve(sph_ctx *ctx, int64_t n);
int sph_sort_and_build(sph_ctx *ctx);          // root box, keys, sort, permute, octree, moments
int sph_tree_refresh_hmax(sph_ctx *ctx);       // cell hmax after h changed
int sph_scan_exclusive(sph_ctx *ctx, const int *in, int *out, const int *len_dev, int len_host, int *total_dev);

// lists (sph_nbr.cu, sph_lists.cu)
int sph_nbr_prepare(sph_ctx *ctx);       // after the sort
int sph_nbr_refresh_h(sph_ctx *ctx);     // after h changed
int sph_build_sph_lists(sph_ctx *ctx, int mode);
int sph_density_from_superset(sph_ctx *ctx);
int sph_density_fused(sph_ctx *ctx);     // mixed precision: all density passes of a step
int sph_nbr_ensure_superset(sph_ctx *ctx);   // mixed precision: density pass without an exact list
int time_mark(sph_ctx *ctx, int seg);
int dl_milestone(sph_ctx *ctx, uint64_t final_fields);   // sph_step_download: send what is final      // event at the end of a timed segment (when timing is on)
int sph_runs_layout(sph_ctx *ctx);        // offsets and tiles of the runs after a change of the run set
int sph_run_reduce_dt(sph_ctx *ctx);      // per-run min dt into runs.dt_dev and runs.dt
int sph_run_diag(sph_ctx *ctx, double *out);   // per-run conserved quantities, out[R * 8]
int sph_build_grav_groups(sph_ctx *ctx);   // gravity i-groups (cells with <= n_group particles)
int sph_build_grav_lists(sph_ctx *ctx);
int sph_gravity_fused(sph_ctx *ctx);       // mixed precision: walk + force in one kernel

// passes (sph_pairs.cu)
int sph_pass_density(sph_ctx *ctx, int build_lists);
int sph_pass_eos(sph_ctx *ctx);
int sph_pass_derivative(sph_ctx *ctx, int build_lists);
int sph_pass_hydro(sph_ctx *ctx, int build_lists);
int sph_pass_gravity(sph_ctx *ctx, int build_lists);
int sph_work_counts(sph_ctx *ctx, int64_t out[8]);
int sph_pack_mixed(sph_ctx *ctx);
int sph_kick_drift_predict(sph_ctx *ctx);   // with each run's dt in runs.dt_dev
int sph_final_kick(sph_ctx *ctx);
int sph_entropy_step(sph_ctx *ctx);       // mode 2: SetConstantEntropy + CalcAll (sph_entropy.cu)
int sph_entropy_check(sph_ctx *ctx);      // fails when the last entropy step had failed lookups
void sph_entropy_free(sph_ctx *ctx);
int sph_ext_force(sph_ctx *ctx);
int sph_diag(sph_ctx *ctx, double out[8]);   // summed over the runs
int sph_init_smth(sph_ctx *ctx, int64_t off, int64_t n);

// ---------------------------------------------------------------------------
// device helpers

static inline int sph_div_up(int64_t a, int64_t b) { return (int)((a + b - 1) / b); }

namespace sph {

// Length argument of the scan kernels: a host value, a device value, or the
// difference of two device values.
struct LenArg {
    const int *p;   // device pointer or null
    int v;          // host value when p is null
    int diff;       // if nonzero, length = p[1] - p[0]
    __device__ int get() const {
        if (!p) return v;
        return diff ? (p[1] - p[0]) : p[0];
    }
};

// Key-and-sort kernels of sph_tree.cu that sph_noalloc.cu also launches.
constexpr int RS_THREADS = 256;          // threads of k_rs_hist / k_rs_scatter (one per digit)
constexpr int RS_ITEMS = 8;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;   // keys per radix-sort tile
__global__ void k_scan_reduce(const int *in, LenArg len, int *part);
__global__ void k_scan_part(int *part, int nb, int *total);
__global__ void k_scan_down(const int *in, int *out, LenArg len, const int *part);
__global__ void k_bbox_partial(const double *x, const double *y, const double *z, int n, double *part);
__global__ void k_bbox_final(const double *part, int nb, double theta, double *rb);
__global__ void k_keys(const double *x, const double *y, const double *z, int n, const double *rb, uint64_t *keys,
                       uint32_t *vals, int *err);
__global__ void k_rs_hist(const uint64_t *keys, int n, int shift, uint32_t *hist, int nb, const int4 *tiles);
__global__ void __launch_bounds__(RS_THREADS) k_rs_scatter(const uint64_t *kin, const uint32_t *vin, uint64_t *kout,
                                                           uint32_t *vout, int n, int shift, const uint32_t *off,
                                                           int nb, const int4 *tiles);

}  // namespace sph

#define FLD(ptr, f, cap) ((ptr) + (int64_t)(f) * (cap))
