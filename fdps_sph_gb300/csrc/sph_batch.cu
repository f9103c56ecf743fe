// Functor-compatible batch entry points (dispatch / retrieve).
//
// These apply the reference functors exactly to caller-supplied walks in the
// class.h payload layouts: RESULT::clear() (class.h:41-85), then for every i
// of the walk the loop over the walk's whole j-list, then the per-i epilogue
// inside the same functor (force.h:18-21, 102-104, 145).  Because the j-list
// is the caller's (an FDPS group superset), out-of-support j contribute zero
// to sums but still enter v_sig_max in the hydro functor, exactly as on the
// CPU.  One CTA per walk; the walk's j-list is staged through shared memory
// in tiles and read by every thread (one thread per i).
//
// Staging: the walks' payloads live in the caller's host memory, one array
// per walk.  Where the GPU can read pageable host memory (GB300's
// NVLink-C2C with the host's page tables), a gather kernel copies every walk
// of a dispatch into the tag's device buffer straight from those arrays over
// the host link, and the dispatch returns once the gather has finished (the
// caller may reuse its arrays after the call, as FDPS does); on retrieve a
// scatter kernel writes the results straight into the caller's RESULT arrays
// the same way.  Otherwise the host copies the walks into pinned staging and
// one host-to-device copy follows, and the results come back through pinned
// memory and are copied to the RESULT arrays by the host.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "sph_batch.cuh"

using namespace sph;

namespace {

std::atomic<int> g_batch_prec{SPH_PREC_FP64};            // the arithmetic of the next dispatches
std::atomic<int> g_batch_staging{SPH_BATCH_STAGING_AUTO};   // who moves the payloads to the device

constexpr int MAX_TAGS = 64;
constexpr int WT = 128;

thread_local std::string g_batch_err;

int batch_fail(int code, const std::string &msg) {
    g_batch_err = msg;
    return code;
}

struct TagState {
    cudaStream_t stream = nullptr;
    char *h_in = nullptr, *d_in = nullptr;      // staged walks
    size_t cap_in = 0;
    char *h_out = nullptr, *d_out = nullptr;    // results
    size_t cap_out = 0;
    int64_t *h_meta = nullptr, *d_meta = nullptr;   // per walk: i offset, n_i, j offset, n_j, s offset, n_s
    size_t cap_meta = 0;
    uint64_t *h_src = nullptr, *d_src = nullptr;    // per walk: the caller's EPI, EPJ, SPJ addresses
    size_t cap_src = 0;
    uint64_t *h_dst = nullptr, *d_dst = nullptr;    // per walk: the caller's RESULT address (retrieve)
    size_t cap_dst = 0;
    cudaEvent_t gathered = nullptr;                 // the device gather of the pending dispatch is done
    bool gather_pending = false;
    bool direct_out = false;                        // results stay on the device until retrieve scatters them
    bool pending_index = false;                     // the pending dispatch is of the index form
    int *d_err = nullptr, *h_err = nullptr;         // index form: bit 0 = an index outside the sent array
    int pageable = -1;                              // the device reads pageable host memory (-1: not asked)
    int pending_kind = -1;
    int pending_walks = 0;
    size_t pending_out_bytes = 0;
    int device = -1;
    std::mutex mu;   // held by one dispatch or retrieve on this tag at a time
};

// Each tag has its own stream, staging and lock: calls on different tags (host threads each
// driving their own tags) stage, launch and wait independently.
TagState g_tags[MAX_TAGS];

std::mutex *tag_mutex(int tag) { return (tag >= 0 && tag < MAX_TAGS) ? &g_tags[tag].mu : nullptr; }

#define SPH_TAG_LOCK(tag)                                                                  \
    std::mutex *tm_ = tag_mutex(tag);                                                       \
    if (!tm_) return batch_fail(SPH_ERR_ARG, "tag out of range [0, 64)");                   \
    std::lock_guard<std::mutex> lk(*tm_)

int grow(char **h, char **d, size_t *cap, size_t need) {
    if (need <= *cap) return SPH_OK;
    size_t c = std::max(need, *cap * 2);
    if (*h) cudaFreeHost(*h);
    if (*d) cudaFree(*d);
    *h = nullptr;
    *d = nullptr;
    *cap = 0;
    if (cudaMallocHost((void **)h, c) != cudaSuccess || cudaMalloc((void **)d, c) != cudaSuccess) {
        cudaGetLastError();
        return batch_fail(SPH_ERR_OOM, "batch staging allocation failed");
    }
    *cap = c;
    return SPH_OK;
}

int tag_state(int tag, TagState **out) {
    if (tag < 0 || tag >= MAX_TAGS) return batch_fail(SPH_ERR_ARG, "tag out of range [0, 64)");
    TagState &t = g_tags[tag];
    int dev = 0;
    cudaGetDevice(&dev);
    if (!t.stream || t.device != dev) {
        if (t.stream) {   // the tag moves to another device: its buffers and stream stay with the old one
            cudaSetDevice(t.device);
            cudaStreamSynchronize(t.stream);
            for (char **h : {&t.h_in, &t.h_out, (char **)&t.h_meta, (char **)&t.h_src, (char **)&t.h_dst,
                             (char **)&t.h_err})
                if (*h) cudaFreeHost(*h);
            for (char **d : {&t.d_in, &t.d_out, (char **)&t.d_meta, (char **)&t.d_src, (char **)&t.d_dst,
                             (char **)&t.d_err})
                if (*d) cudaFree(*d);
            cudaStreamDestroy(t.stream);
            if (t.gathered) cudaEventDestroy(t.gathered);
            cudaSetDevice(dev);
            t.h_in = t.h_out = t.d_in = t.d_out = nullptr;
            t.h_meta = t.d_meta = nullptr;
            t.h_src = t.d_src = t.h_dst = t.d_dst = nullptr;
            t.h_err = t.d_err = nullptr;
            t.cap_in = t.cap_out = t.cap_meta = t.cap_src = t.cap_dst = 0;
            t.stream = nullptr;
            t.gathered = nullptr;
            t.pending_kind = -1;
            t.gather_pending = false;
        }
        if (cudaStreamCreateWithFlags(&t.stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&t.gathered, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            return batch_fail(SPH_ERR_CUDA, "cannot create a CUDA stream (no GPU?)");
        }
        t.device = dev;
        t.pageable = -1;
    }
    *out = &t;
    return SPH_OK;
}

// ---------------------------------------------------------------------------
// kernels: meta[w*6 + {0..5}] = i offset, n_i, j offset, n_j, spj offset, n_spj (element offsets)

__device__ __forceinline__ double3 ld3(const double *p) { return make_double3(p[0], p[1], p[2]); }

static_assert(sizeof(sph_epi_dens) % 8 == 0 && sizeof(sph_epj_dens) % 8 == 0 && sizeof(sph_epi_drvt) % 8 == 0 &&
                  sizeof(sph_epj_drvt) % 8 == 0 && sizeof(sph_epi_hydro) % 8 == 0 &&
                  sizeof(sph_epj_hydro) % 8 == 0 && sizeof(sph_epi_grav) % 8 == 0 &&
                  sizeof(sph_epj_grav) % 8 == 0 && sizeof(sph_spj_monopole) % 8 == 0,
              "payloads move as 8-byte words");

static_assert(sizeof(sph_result_dens) % 8 == 0 && sizeof(sph_result_drvt) % 8 == 0 &&
                  sizeof(sph_result_hydro) % 8 == 0 && sizeof(sph_result_grav) % 8 == 0,
              "results move as 8-byte words");

// a block copies n 8-byte words, four independent loads per thread in flight (the source may be
// host memory across the host link, where the latency wants many loads outstanding)
__device__ __forceinline__ void copy_words(const unsigned long long *src, unsigned long long *dst, int64_t n) {
    const int64_t bd = blockDim.x;
    int64_t k = threadIdx.x;
    for (; k + 3 * bd < n; k += 4 * bd) {
        const unsigned long long a = src[k], b = src[k + bd], c = src[k + 2 * bd], d = src[k + 3 * bd];
        dst[k] = a;
        dst[k + bd] = b;
        dst[k + 2 * bd] = c;
        dst[k + 3 * bd] = d;
    }
    for (; k < n; k += bd) dst[k] = src[k];
}

// the same in 4-byte words (the index form's int32 index arrays)
__device__ __forceinline__ void copy_words4(const unsigned *src, unsigned *dst, int64_t n) {
    const int64_t bd = blockDim.x;
    int64_t k = threadIdx.x;
    for (; k + 3 * bd < n; k += 4 * bd) {
        const unsigned a = src[k], b = src[k + bd], c = src[k + 2 * bd], d = src[k + 3 * bd];
        dst[k] = a;
        dst[k + bd] = b;
        dst[k + 2 * bd] = c;
        dst[k + 3 * bd] = d;
    }
    for (; k < n; k += bd) dst[k] = src[k];
}

// a run of `bytes` bytes in 8-byte words, or in 4-byte words where the element size is not a
// multiple of 8 (the host checked the alignment)
__device__ __forceinline__ void copy_run(const void *src, void *dst, int64_t bytes, int elem) {
    if (elem % 8 == 0) copy_words((const unsigned long long *)src, (unsigned long long *)dst, bytes / 8);
    else copy_words4((const unsigned *)src, (unsigned *)dst, bytes / 4);
}

// block w copies walk w's EPI, EPJ and SPJ runs (payloads, or index arrays in the index form) from
// the caller's arrays (host memory, read over the host link) to their places in the tag's device
// staging; s_* are the element sizes in bytes
__global__ void __launch_bounds__(256) k_gather_walks(const int64_t *meta, const uint64_t *src, char *dst,
                                                      int64_t o_epj, int64_t o_spj, int s_epi, int s_epj,
                                                      int s_spj) {
    const int64_t *m = meta + 6 * blockIdx.x;
    const uint64_t *p = src + 3 * blockIdx.x;
    if (m[1] > 0) copy_run((const void *)p[0], dst + (int64_t)s_epi * m[0], (int64_t)s_epi * m[1], s_epi);
    if (m[3] > 0) copy_run((const void *)p[1], dst + o_epj + (int64_t)s_epj * m[2], (int64_t)s_epj * m[3], s_epj);
    if (m[5] > 0) copy_run((const void *)p[2], dst + o_spj + (int64_t)s_spj * m[4], (int64_t)s_spj * m[5], s_spj);
}

// block w copies walk w's results from the tag's device buffer to the caller's RESULT array
__global__ void __launch_bounds__(256) k_scatter_results(const int64_t *meta, const uint64_t *dst, const char *src,
                                                         int s_res) {
    const int64_t *m = meta + 6 * blockIdx.x;
    if (m[1] > 0)
        copy_words((const unsigned long long *)(src + (int64_t)s_res * m[0]), (unsigned long long *)dst[blockIdx.x],
                   (int64_t)s_res * m[1] / 8);
}

// CalcDensity, force.h:9-23
__global__ void __launch_bounds__(WT) k_walk_dens(const int64_t *meta, const sph_epi_dens *epi, JSrc<sph_epj_dens> epj,
                                                  sph_result_dens *res) {
    __shared__ double4 tile[WT];
    const int64_t *M = meta + 6 * blockIdx.x;
    const int64_t io = M[0], ni = M[1], jo = M[2], nj = M[3];
    for (int64_t i0 = 0; i0 < ni; i0 += WT) {
        const int64_t ii = i0 + threadIdx.x;
        const bool act = ii < ni;
        double3 pi = make_double3(0, 0, 0);
        double hi = 1.0, mi = 1.0;
        if (act) {
            pi = ld3(epi[io + ii].pos);
            hi = epi[io + ii].smth;
            mi = epi[io + ii].mass;
        }
        const double H = SUPPORT * hi, invH = 1.0 / H, norm = kernel_norm(H);
        double d = 0.0;
        for (int64_t t0 = 0; t0 < nj; t0 += WT) {
            if (t0 + threadIdx.x < nj) {
                const sph_epj_dens &q = epj[jo + t0 + threadIdx.x];
                tile[threadIdx.x] = make_double4(q.pos[0], q.pos[1], q.pos[2], q.mass);
            }
            __syncthreads();
            const int tn = (int)min((int64_t)WT, nj - t0);
            for (int t = 0; t < tn; ++t) {
                const double4 q = tile[t];
                const double dx = q.x - pi.x, dy = q.y - pi.y, dz = q.z - pi.z;
                double w, g;
                wendland_poly(sqrt(dx * dx + dy * dy + dz * dz) * invH, w, g);
                d += q.w * (w * norm);
            }
            __syncthreads();
        }
        if (act) {
            d = fmax(DENS_FLOOR, d);
            res[io + ii].dens = d;
            res[io + ii].smth = SMTH_COEF * pow(mi / d, 1.0 / 3.0);
        }
    }
}

// CalcDerivative, force.h:89-106
__global__ void __launch_bounds__(WT) k_walk_drvt(const int64_t *meta, const sph_epi_drvt *epi, JSrc<sph_epj_drvt> epj,
                                                  sph_result_drvt *res) {
    __shared__ double4 tp[WT];
    __shared__ double4 tv[WT];
    const int64_t *M = meta + 6 * blockIdx.x;
    const int64_t io = M[0], ni = M[1], jo = M[2], nj = M[3];
    for (int64_t i0 = 0; i0 < ni; i0 += WT) {
        const int64_t ii = i0 + threadIdx.x;
        const bool act = ii < ni;
        double3 pi = make_double3(0, 0, 0), vi = make_double3(0, 0, 0);
        double hi = 1.0, rhoi = 1.0;
        if (act) {
            pi = ld3(epi[io + ii].pos);
            vi = ld3(epi[io + ii].vel);
            hi = epi[io + ii].smth;
            rhoi = epi[io + ii].dens;
        }
        const double H = SUPPORT * hi, invH = 1.0 / H, norm = kernel_norm(H), ceps = 1.0e-6 * hi;
        double dv = 0, r0 = 0, r1 = 0, r2 = 0, gs = 0;
        for (int64_t t0 = 0; t0 < nj; t0 += WT) {
            if (t0 + threadIdx.x < nj) {
                const sph_epj_drvt &q = epj[jo + t0 + threadIdx.x];
                tp[threadIdx.x] = make_double4(q.pos[0], q.pos[1], q.pos[2], q.mass);
                tv[threadIdx.x] = make_double4(q.vel[0], q.vel[1], q.vel[2], 0.0);
            }
            __syncthreads();
            const int tn = (int)min((int64_t)WT, nj - t0);
            for (int t = 0; t < tn; ++t) {
                const double4 q = tp[t], u = tv[t];
                const double dx = pi.x - q.x, dy = pi.y - q.y, dz = pi.z - q.z;
                const double ax = -q.w * (vi.x - u.x), ay = -q.w * (vi.y - u.y), az = -q.w * (vi.z - u.z);
                const double rr2 = dx * dx + dy * dy + dz * dz;
                const double r = sqrt(rr2);
                double w, g;
                wendland_poly(r * invH, w, g);
                const double gf = norm * g / (r * H + ceps);
                dv += gf * (ax * dx + ay * dy + az * dz);
                r0 += gf * (ay * dz - az * dy);
                r1 += gf * (az * dx - ax * dz);
                r2 += gf * (ax * dy - ay * dx);
                gs -= q.w / hi * (3.0 * norm * w + gf * rr2);
            }
            __syncthreads();
        }
        if (act) {
            sph_result_drvt &o = res[io + ii];
            o.grad_smth = 1.0 / (1.0 + hi * gs / (3.0 * rhoi));
            o.div_v = dv / rhoi;
            o.rot_v[0] = r0 / rhoi;
            o.rot_v[1] = r1 / rhoi;
            o.rot_v[2] = r2 / rhoi;
        }
    }
}

// CalcHydroForce, force.h:113-147
__global__ void __launch_bounds__(WT) k_walk_hydro(const int64_t *meta, const sph_epi_hydro *epi,
                                                   JSrc<sph_epj_hydro> epj, sph_result_hydro *res) {
    __shared__ double4 tp[WT];   // pos, mass
    __shared__ double4 tv[WT];   // vel, smth
    __shared__ double4 tq[WT];   // dens, pres, snds, grad_smth
    __shared__ double tb[WT];    // Bal
    const int64_t *M = meta + 6 * blockIdx.x;
    const int64_t io = M[0], ni = M[1], jo = M[2], nj = M[3];
    for (int64_t i0 = 0; i0 < ni; i0 += WT) {
        const int64_t ii = i0 + threadIdx.x;
        const bool act = ii < ni;
        sph_epi_hydro I;
        if (act) I = epi[io + ii];
        else std::memset(&I, 0, sizeof(I)), I.smth = 1.0, I.dens = 1.0;
        const double Hi = SUPPORT * I.smth, invHi = 1.0 / Hi, normi = kernel_norm(Hi), cepsi = 1.0e-6 * I.smth;
        const double Ai = I.grad_smth * I.pres / (I.dens * I.dens);
        double a0 = 0, a1 = 0, a2 = 0, e = 0, vmax = 0.0;
        for (int64_t t0 = 0; t0 < nj; t0 += WT) {
            if (t0 + threadIdx.x < nj) {
                const sph_epj_hydro &q = epj[jo + t0 + threadIdx.x];
                tp[threadIdx.x] = make_double4(q.pos[0], q.pos[1], q.pos[2], q.mass);
                tv[threadIdx.x] = make_double4(q.vel[0], q.vel[1], q.vel[2], q.smth);
                tq[threadIdx.x] = make_double4(q.dens, q.pres, q.snds, q.grad_smth);
                tb[threadIdx.x] = q.Bal;
            }
            __syncthreads();
            const int tn = (int)min((int64_t)WT, nj - t0);
            for (int t = 0; t < tn; ++t) {
                const double4 p = tp[t], v = tv[t], q = tq[t];
                const double dx = I.pos[0] - p.x, dy = I.pos[1] - p.y, dz = I.pos[2] - p.z;
                const double wx = I.vel[0] - v.x, wy = I.vel[1] - v.y, wz = I.vel[2] - v.z;
                const double rr2 = dx * dx + dy * dy + dz * dz;
                const double r = sqrt(rr2);
                const double dvdr = wx * dx + wy * dy + wz * dz;
                const double w = (dvdr < 0) ? dvdr / r : 0.0;
                const double vsig = I.snds + q.z - 3.0 * w;
                vmax = fmax(vmax, vsig);
                const double AV = -AV_STRENGTH * 0.5 * vsig * w / (0.5 * (I.dens + q.x)) * 0.5 * (I.Bal + tb[t]);
                const double Hj = SUPPORT * v.w;
                double wi_, gi_, wj_, gj_;
                wendland_poly(r * invHi, wi_, gi_);
                wendland_poly(r / Hj, wj_, gj_);
                const double gfi = normi * gi_ / (r * Hi + cepsi);
                const double gfj = kernel_norm(Hj) * gj_ / (r * Hj + 1.0e-6 * v.w);
                const double gws = 0.5 * (gfi * I.grad_smth + gfj * q.w);
                const double Aj = q.w * q.y / (q.x * q.x);
                const double coef = p.w * (Ai * gfi + Aj * gfj + AV * gws);
                a0 -= coef * dx;
                a1 -= coef * dy;
                a2 -= coef * dz;
                e += p.w * (Ai + 0.5 * AV) * gws * dvdr;
            }
            __syncthreads();
        }
        if (act) {
            sph_result_hydro &o = res[io + ii];
            o.acc[0] = a0;
            o.acc[1] = a1;
            o.acc[2] = a2;
            o.eng_dot = e;
            o.dt = C_CFL * 2.0 * I.smth / vmax;
        }
    }
}

// CalcGravityForce<EPJ::Grav> then CalcGravityForce<SPJMonopole>, force.h:154-168
__global__ void __launch_bounds__(WT) k_walk_grav(const int64_t *meta, const sph_epi_grav *epi, JSrc<sph_epj_grav> epj,
                                                  JSrc<sph_spj_monopole> spj, sph_result_grav *res) {
    __shared__ double4 tile[WT];
    const double G = 6.67e-11;   // force.h:171-172
    const int64_t *M = meta + 6 * blockIdx.x;
    const int64_t io = M[0], ni = M[1], jo = M[2], nj = M[3], so = M[4], ns = M[5];
    for (int64_t i0 = 0; i0 < ni; i0 += WT) {
        const int64_t ii = i0 + threadIdx.x;
        const bool act = ii < ni;
        double3 pi = make_double3(0, 0, 0);
        double eps2 = 1.0;
        if (act) {
            pi = ld3(epi[io + ii].pos);
            eps2 = epi[io + ii].eps2;
        }
        double a0 = 0, a1 = 0, a2 = 0, p = 0;
        for (int pass = 0; pass < 2; ++pass) {
            const int64_t nl = pass == 0 ? nj : ns;
            for (int64_t t0 = 0; t0 < nl; t0 += WT) {
                if (t0 + threadIdx.x < nl) {
                    if (pass == 0) {
                        const sph_epj_grav &q = epj[jo + t0 + threadIdx.x];
                        tile[threadIdx.x] = make_double4(q.pos[0], q.pos[1], q.pos[2], q.mass);
                    } else {
                        const sph_spj_monopole &q = spj[so + t0 + threadIdx.x];
                        tile[threadIdx.x] = make_double4(q.pos[0], q.pos[1], q.pos[2], q.mass);
                    }
                }
                __syncthreads();
                const int tn = (int)min((int64_t)WT, nl - t0);
                for (int t = 0; t < tn; ++t) {
                    const double4 q = tile[t];
                    const double dx = pi.x - q.x, dy = pi.y - q.y, dz = pi.z - q.z;
                    const double dri = 1.0 / sqrt(dx * dx + dy * dy + dz * dz + eps2);
                    const double mdr3 = q.w * (dri * dri * dri);
                    a0 -= G * mdr3 * dx;
                    a1 -= G * mdr3 * dy;
                    a2 -= G * mdr3 * dz;
                    p -= G * q.w * dri;
                }
                __syncthreads();
            }
        }
        if (act) {
            sph_result_grav &o = res[io + ii];
            o.acc[0] = a0;
            o.acc[1] = a1;
            o.acc[2] = a2;
            o.pot = p;
            o.dt = 1.0e30;   // RESULT::Grav::clear(), dt untouched by the functor
        }
    }
}

// where a dispatch's sections sit in the tag's staging (bytes, 16-byte aligned sections)
struct Layout {
    int64_t ni = 0, nj = 0, ns = 0;
    size_t o_epj = 0, o_spj = 0, end = 0;
};

// Stages one dispatch's walks on its tag: the EPI payloads, then the j entries of every walk and
// (gravity) its SPJ entries.  Payload form: the entries are EPJ / SPJ payloads (s_j, s_s their
// sizes); index form: int32 indices into the arrays sent for the pass (s_j = s_s = 4).
template <class EPI, class RES>
int stage(int tag, int kind, int n_walk, const EPI **epi, const int *n_epi, const void *const *jw, size_t s_j,
          const int *n_epj, const void *const *sw, size_t s_s, const int *n_spj, bool index, TagState **ts_out,
          Layout *lay) {
    if (n_walk < 0 || (n_walk > 0 && (!epi || !n_epi || !jw || !n_epj)))
        return batch_fail(SPH_ERR_ARG, "null walk arrays");
    TagState *ts = nullptr;
    SPH_TRY(tag_state(tag, &ts));
    if (ts->pending_kind >= 0) {
        // a previous dispatch on this tag was never retrieved: finish it first
        cudaStreamSynchronize(ts->stream);
        ts->pending_kind = -1;
    }
    Layout L;
    for (int w = 0; w < n_walk; ++w) {
        if (n_epi[w] < 0 || n_epj[w] < 0 || (sw && n_spj && n_spj[w] < 0))
            return batch_fail(SPH_ERR_ARG, "negative walk size");
        if ((n_epi[w] > 0 && !epi[w]) || (n_epj[w] > 0 && !jw[w])) return batch_fail(SPH_ERR_ARG, "null walk");
        L.ni += n_epi[w];
        L.nj += n_epj[w];
        if (sw && n_spj) L.ns += n_spj[w];
    }
    const size_t b_epi = sizeof(EPI) * L.ni, b_epj = s_j * L.nj, b_spj = s_s * L.ns;
    L.o_epj = (b_epi + 15) & ~size_t(15);
    L.o_spj = (L.o_epj + b_epj + 15) & ~size_t(15);
    L.end = L.o_spj + b_spj;
    SPH_TRY(grow(&ts->h_in, &ts->d_in, &ts->cap_in, L.end + 16));
    SPH_TRY(grow(&ts->h_out, &ts->d_out, &ts->cap_out, sizeof(RES) * L.ni + 16));
    SPH_TRY(grow((char **)&ts->h_meta, (char **)&ts->d_meta, &ts->cap_meta, sizeof(int64_t) * 6 * (n_walk + 1)));
    if (index && !ts->d_err) {
        if (cudaMalloc((void **)&ts->d_err, sizeof(int)) != cudaSuccess ||
            cudaMallocHost((void **)&ts->h_err, sizeof(int)) != cudaSuccess) {
            cudaGetLastError();
            return batch_fail(SPH_ERR_OOM, "batch error-word allocation failed");
        }
    }
    int64_t ai = 0, aj = 0, as = 0;
    for (int w = 0; w < n_walk; ++w) {
        int64_t *m = ts->h_meta + 6 * w;
        m[0] = ai;
        m[1] = n_epi[w];
        m[2] = aj;
        m[3] = n_epj[w];
        m[4] = as;
        m[5] = (sw && n_spj) ? n_spj[w] : 0;
        if (m[5] && !sw[w]) return batch_fail(SPH_ERR_ARG, "null SPJ walk");
        ai += n_epi[w];
        aj += n_epj[w];
        as += m[5];
    }
    // who moves the payloads: the device gather where this GPU reads pageable host memory and every
    // array is aligned to its word (8 bytes for payloads, 4 for indices), else the host
    const int mode = g_batch_staging.load();
    bool gather = false;
    if (mode != SPH_BATCH_STAGING_HOST && n_walk > 0) {
        if (ts->pageable < 0) {
            int v = 0;
            if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, ts->device) != cudaSuccess) {
                cudaGetLastError();
                v = 0;
            }
            ts->pageable = v == 1;
        }
        gather = ts->pageable == 1;
        const uintptr_t aj_mask = s_j % 8 ? 3u : 7u, as_mask = s_s % 8 ? 3u : 7u;
        for (int w = 0; gather && w < n_walk; ++w) {
            const int64_t *m = ts->h_meta + 6 * w;
            gather = !(m[1] && ((uintptr_t)epi[w] & 7u)) && !(m[3] && ((uintptr_t)jw[w] & aj_mask)) &&
                     !(m[5] && ((uintptr_t)sw[w] & as_mask));
        }
        if (!gather && mode == SPH_BATCH_STAGING_DEVICE)
            return batch_fail(SPH_ERR_STATE, ts->pageable == 1
                                                 ? "SPH_BATCH_STAGING_DEVICE needs word-aligned walk arrays"
                                                 : "this GPU cannot read pageable host memory "
                                                   "(SPH_BATCH_STAGING_DEVICE)");
    }
    if (index && cudaMemsetAsync(ts->d_err, 0, sizeof(int), ts->stream) != cudaSuccess) {
        cudaGetLastError();
        return batch_fail(SPH_ERR_CUDA, "cannot clear the batch error word");
    }
    if (gather) {
        SPH_TRY(grow((char **)&ts->h_src, (char **)&ts->d_src, &ts->cap_src, sizeof(uint64_t) * 3 * (n_walk + 1)));
        for (int w = 0; w < n_walk; ++w) {
            const int64_t *m = ts->h_meta + 6 * w;
            ts->h_src[3 * w] = m[1] ? (uint64_t)(uintptr_t)epi[w] : 0;
            ts->h_src[3 * w + 1] = m[3] ? (uint64_t)(uintptr_t)jw[w] : 0;
            ts->h_src[3 * w + 2] = m[5] ? (uint64_t)(uintptr_t)sw[w] : 0;
        }
        if (cudaMemcpyAsync(ts->d_meta, ts->h_meta, sizeof(int64_t) * 6 * n_walk, cudaMemcpyHostToDevice,
                            ts->stream) != cudaSuccess ||
            cudaMemcpyAsync(ts->d_src, ts->h_src, sizeof(uint64_t) * 3 * n_walk, cudaMemcpyHostToDevice,
                            ts->stream) != cudaSuccess) {
            cudaGetLastError();
            return batch_fail(SPH_ERR_CUDA, "host-to-device copy failed");
        }
        k_gather_walks<<<n_walk, 256, 0, ts->stream>>>(ts->d_meta, ts->d_src, ts->d_in, (int64_t)L.o_epj,
                                                       (int64_t)L.o_spj, (int)sizeof(EPI), (int)s_j, (int)s_s);
        if (cudaGetLastError() != cudaSuccess || cudaEventRecord(ts->gathered, ts->stream) != cudaSuccess) {
            cudaGetLastError();
            return batch_fail(SPH_ERR_CUDA, "walk gather launch failed");
        }
        ts->gather_pending = true;
        ts->direct_out = true;
    } else {
        ts->direct_out = false;
        // the walks' payloads into the pinned staging, split over the host threads (a dispatch of a
        // few hundred walks moves hundreds of MB; one thread copies at a fraction of the memory
        // bandwidth).  Inside a caller's own parallel region (FDPS's OpenMP threads) this runs on
        // the calling thread.
#pragma omp parallel for schedule(dynamic, 4) if (n_walk > 8 && ai + aj > 65536)
        for (int w = 0; w < n_walk; ++w) {
            const int64_t *m = ts->h_meta + 6 * w;
            if (m[1]) std::memcpy(ts->h_in + sizeof(EPI) * m[0], epi[w], sizeof(EPI) * m[1]);
            if (m[3]) std::memcpy(ts->h_in + L.o_epj + s_j * m[2], jw[w], s_j * m[3]);
            if (m[5]) std::memcpy(ts->h_in + L.o_spj + s_s * m[4], sw[w], s_s * m[5]);
        }
        if (cudaMemcpyAsync(ts->d_in, ts->h_in, L.end, cudaMemcpyHostToDevice, ts->stream) != cudaSuccess ||
            cudaMemcpyAsync(ts->d_meta, ts->h_meta, sizeof(int64_t) * 6 * n_walk, cudaMemcpyHostToDevice,
                            ts->stream) != cudaSuccess) {
            cudaGetLastError();
            return batch_fail(SPH_ERR_CUDA, "host-to-device copy failed");
        }
    }
    ts->pending_kind = kind;
    ts->pending_index = index;
    ts->pending_walks = n_walk;
    ts->pending_out_bytes = sizeof(RES) * L.ni;
    *ts_out = ts;
    *lay = L;
    return SPH_OK;
}

int finish_dispatch(TagState *ts) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return batch_fail(SPH_ERR_CUDA, std::string("kernel launch failed: ") + cudaGetErrorString(e));
    if (!ts->direct_out && ts->pending_out_bytes &&
        cudaMemcpyAsync(ts->h_out, ts->d_out, ts->pending_out_bytes, cudaMemcpyDeviceToHost, ts->stream) != cudaSuccess) {
        cudaGetLastError();
        return batch_fail(SPH_ERR_CUDA, "device-to-host copy failed");
    }
    if (ts->gather_pending) {   // the caller may reuse its walk arrays once the call returns
        ts->gather_pending = false;
        const cudaError_t g = cudaEventSynchronize(ts->gathered);
        if (g != cudaSuccess) return batch_fail(SPH_ERR_CUDA, std::string("walk gather failed: ") + cudaGetErrorString(g));
    }
    return SPH_OK;
}

// ---------------------------------------------------------------------------
// index form: the EPJ (and SPJ) arrays of a pass, sent once and kept on the device

struct Resident {
    char *d_j = nullptr, *d_s = nullptr;
    size_t cap_j = 0, cap_s = 0;
    int64_t n_j = 0, n_s = 0;
    int device = -1;
    cudaStream_t stream = nullptr;   // the copies of a send (non-blocking: independent of other work)
    int pageable = -1;               // the device reads pageable host memory (-1: not asked)
    std::mutex mu;
};
Resident g_res[4];   // per kind: density, derivative, hydro, gravity

// a flat copy in 8-byte words by the whole grid, four loads per thread in flight
__global__ void __launch_bounds__(256) k_copy_flat(const unsigned long long *src, unsigned long long *dst, int64_t n) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    for (; k + 3 * stride < n; k += 4 * stride) {
        const unsigned long long a = src[k], b = src[k + stride], c = src[k + 2 * stride], d = src[k + 3 * stride];
        dst[k] = a;
        dst[k + stride] = b;
        dst[k + 2 * stride] = c;
        dst[k + 3 * stride] = d;
    }
    for (; k < n; k += stride) dst[k] = src[k];
}

// one sent array to the device: read by the GPU straight from the caller's memory where it can
// read pageable host memory, the array is 8-byte aligned and the staging is not forced to the host
// (NVLink-C2C, about 200 GB/s), else cudaMemcpy; returns after the copy
int upload_array(Resident &R, char *dst, const void *src, size_t bytes) {
    if (bytes == 0) return SPH_OK;
    if (R.pageable == 1 && g_batch_staging.load() != SPH_BATCH_STAGING_HOST && bytes % 8 == 0 &&
        ((uintptr_t)src & 7u) == 0) {
        const int64_t words = (int64_t)(bytes / 8);
        const int grid = (int)std::min<int64_t>(152 * 8, (words + 255) / 256);
        k_copy_flat<<<grid, 256, 0, R.stream>>>((const unsigned long long *)src, (unsigned long long *)dst, words);
        if (cudaGetLastError() == cudaSuccess && cudaStreamSynchronize(R.stream) == cudaSuccess) return SPH_OK;
        cudaGetLastError();
        return batch_fail(SPH_ERR_CUDA, "copy of a sent EPJ / SPJ array failed");
    }
    if (cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaGetLastError();
        return batch_fail(SPH_ERR_CUDA, "copy of a sent EPJ / SPJ array failed");
    }
    return SPH_OK;
}

int grow_dev(char **d, size_t *cap, size_t need) {
    if (need <= *cap) return SPH_OK;
    const size_t c = std::max(need, *cap + *cap / 2);
    if (*d) cudaFree(*d);
    *d = nullptr;
    *cap = 0;
    if (cudaMalloc((void **)d, c) != cudaSuccess) {
        cudaGetLastError();
        return batch_fail(SPH_ERR_OOM, "allocation of the sent EPJ / SPJ arrays failed");
    }
    *cap = c;
    return SPH_OK;
}

// send_flag: the pass's whole EPJ array (and SPJ array) to the device.  Index dispatches of this
// kind already issued may still read the previous arrays: their tags' streams are waited for first
// (tag by tag, one lock at a time).  Returns after the copy, so the caller may reuse its arrays.
int send_resident(int kind, const void *a, int64_t n, size_t sa, const void *b, int64_t nb, size_t sb) {
    if (n < 0 || nb < 0 || (n > 0 && !a) || (nb > 0 && !b)) return batch_fail(SPH_ERR_ARG, "bad EPJ / SPJ array");
    for (int t = 0; t < MAX_TAGS; ++t) {
        std::lock_guard<std::mutex> lk(g_tags[t].mu);
        if (g_tags[t].pending_kind == kind && g_tags[t].pending_index) cudaStreamSynchronize(g_tags[t].stream);
    }
    Resident &R = g_res[kind];
    std::lock_guard<std::mutex> lk(R.mu);
    int dev = 0;
    cudaGetDevice(&dev);
    if (R.device != dev) {   // buffers of another device are dropped
        if (R.device >= 0 && (R.d_j || R.d_s)) {
            cudaSetDevice(R.device);
            if (R.d_j) cudaFree(R.d_j);
            if (R.d_s) cudaFree(R.d_s);
            cudaSetDevice(dev);
        }
        R.d_j = R.d_s = nullptr;
        R.cap_j = R.cap_s = 0;
        R.stream = nullptr;   // a stream of the other device is left to it
        R.device = dev;
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess) {
            cudaGetLastError();
            v = 0;
        }
        R.pageable = v == 1;
    }
    if (!R.stream && cudaStreamCreateWithFlags(&R.stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        R.stream = nullptr;
        return batch_fail(SPH_ERR_CUDA, "cannot create a CUDA stream (no GPU?)");
    }
    R.n_j = R.n_s = 0;
    SPH_TRY(grow_dev(&R.d_j, &R.cap_j, sa * (size_t)n + 16));
    SPH_TRY(grow_dev(&R.d_s, &R.cap_s, sb * (size_t)nb + 16));
    SPH_TRY(upload_array(R, R.d_j, a, sa * (size_t)n));
    SPH_TRY(upload_array(R, R.d_s, b, sb * (size_t)nb));
    R.n_j = n;
    R.n_s = nb;
    return SPH_OK;
}

// the sent arrays of a kind, as the index walks' j sources (their error word is the tag's, set
// after staging); walks with entries need a sent array.  Checked before anything is staged, so a
// refused dispatch leaves nothing reading the caller's arrays.
template <class EPJ, class SPJ>
int resident_src(int kind, int n_walk, const int *n_epj, const int *n_spj, JSrc<EPJ> *js, JSrc<SPJ> *ss) {
    Resident &R = g_res[kind];
    std::lock_guard<std::mutex> lk(R.mu);
    int dev = 0;
    cudaGetDevice(&dev);
    bool need_j = false, need_s = false;
    for (int w = 0; w < n_walk && n_epj; ++w) {
        need_j = need_j || n_epj[w] > 0;
        need_s = need_s || (n_spj && n_spj[w] > 0);
    }
    if ((need_j && (R.n_j == 0 || R.device != dev)) || (need_s && (R.n_s == 0 || R.device != dev)))
        return batch_fail(SPH_ERR_STATE, "index walks before their EPJ / SPJ array was sent (send_flag)");
    *js = JSrc<EPJ>{(const EPJ *)R.d_j, nullptr, R.n_j, nullptr};
    if (ss) *ss = JSrc<SPJ>{(const SPJ *)R.d_s, nullptr, R.n_s, nullptr};
    return SPH_OK;
}

template <class RES>
int retrieve(int tag, int kind, int n_walk, const int *n_epi, RES **result) {
    SPH_TAG_LOCK(tag);
    TagState &ts = g_tags[tag];
    if (n_walk == 0 && ts.pending_kind < 0) return SPH_OK;   // nothing was dispatched (a send-only call)
    if (ts.pending_kind != kind || ts.pending_walks != n_walk)
        return batch_fail(SPH_ERR_STATE, "retrieve does not match the last dispatch on this tag");
    std::vector<int64_t> off(n_walk + 1, 0);
    bool bad = false, aligned = true;
    for (int w = 0; w < n_walk; ++w) {
        bad = bad || (n_epi[w] > 0 && (!result || !result[w])) || n_epi[w] != ts.h_meta[6 * w + 1];
        aligned = aligned && !(n_epi[w] > 0 && result && ((uintptr_t)result[w] & 7u));
        off[w + 1] = off[w] + std::max(n_epi[w], 0);
    }
    if (bad) {   // the results are dropped with the dispatch
        cudaStreamSynchronize(ts.stream);
        ts.pending_kind = -1;
        return batch_fail(SPH_ERR_ARG, "null result pointer, or walk sizes that differ from the dispatch's");
    }
    const bool index = ts.pending_index;
    if (index) cudaMemcpyAsync(ts.h_err, ts.d_err, sizeof(int), cudaMemcpyDeviceToHost, ts.stream);
    auto index_check = [&]() {
        return (index && *ts.h_err) ? batch_fail(SPH_ERR_ARG, "an index walk names an entry outside the sent array")
                                    : SPH_OK;
    };
    if (ts.direct_out && aligned && n_walk > 0) {
        // the scatter kernel writes every walk's results into the caller's arrays
        const int rc = grow((char **)&ts.h_dst, (char **)&ts.d_dst, &ts.cap_dst, sizeof(uint64_t) * (n_walk + 1));
        if (rc != SPH_OK) {
            cudaStreamSynchronize(ts.stream);
            ts.pending_kind = -1;
            return rc;
        }
        for (int w = 0; w < n_walk; ++w) ts.h_dst[w] = n_epi[w] > 0 ? (uint64_t)(uintptr_t)result[w] : 0;
        if (cudaMemcpyAsync(ts.d_dst, ts.h_dst, sizeof(uint64_t) * n_walk, cudaMemcpyHostToDevice, ts.stream) ==
            cudaSuccess)
            k_scatter_results<<<n_walk, 256, 0, ts.stream>>>(ts.d_meta, ts.d_dst, ts.d_out, (int)sizeof(RES));
        const cudaError_t e = cudaStreamSynchronize(ts.stream);
        ts.pending_kind = -1;
        const cudaError_t l = cudaGetLastError();
        if (e != cudaSuccess || l != cudaSuccess)
            return batch_fail(SPH_ERR_CUDA, std::string("batch kernel or result scatter failed: ") +
                                                 cudaGetErrorString(e != cudaSuccess ? e : l));
        return index_check();
    }
    if (ts.direct_out && ts.pending_out_bytes)   // results left on the device: bring them to the host now
        cudaMemcpyAsync(ts.h_out, ts.d_out, ts.pending_out_bytes, cudaMemcpyDeviceToHost, ts.stream);
    const cudaError_t e = cudaStreamSynchronize(ts.stream);
    ts.pending_kind = -1;
    const cudaError_t l = cudaGetLastError();
    if (e != cudaSuccess || l != cudaSuccess)
        return batch_fail(SPH_ERR_CUDA, std::string("batch kernel failed: ") +
                                             cudaGetErrorString(e != cudaSuccess ? e : l));
#pragma omp parallel for schedule(dynamic, 8) if (n_walk > 8 && off[n_walk] > 65536)
    for (int w = 0; w < n_walk; ++w)
        if (n_epi[w] > 0) std::memcpy(result[w], ts.h_out + sizeof(RES) * off[w], sizeof(RES) * n_epi[w]);
    return index_check();
}

// one dispatch of a kind, payload or index form: stage, launch the functor kernel, start the
// result copy
template <class EPI, class EPJ, class RES, class LAUNCH>
int dispatch_walks(int tag, int kind, int n_walk, const EPI **epi, const int *n_epi, const void *const *jw,
                   const int *n_epj, bool index, LAUNCH launch) {
    SPH_TAG_LOCK(tag);
    TagState *ts = nullptr;
    Layout L;
    JSrc<EPJ> rj{};
    if (index) SPH_TRY((resident_src<EPJ, sph_spj_monopole>(kind, n_walk, n_epj, nullptr, &rj, nullptr)));
    SPH_TRY((stage<EPI, RES>(tag, kind, n_walk, epi, n_epi, jw, index ? sizeof(int) : sizeof(EPJ), n_epj, nullptr, 0,
                             nullptr, index, &ts, &L)));
    // from here on the dispatch runs to finish_dispatch, which waits for a device gather
    if (n_walk > 0) {
        JSrc<EPJ> js{(const EPJ *)(ts->d_in + L.o_epj), nullptr, 0, nullptr};
        if (index) js = JSrc<EPJ>{rj.base, (const int *)(ts->d_in + L.o_epj), rj.n, ts->d_err};
        launch(ts, (const EPI *)ts->d_in, js, (RES *)ts->d_out, g_batch_prec.load() == SPH_PREC_MIXED);
    }
    return finish_dispatch(ts);
}

int dispatch_grav(int tag, int n_walk, const sph_epi_grav **epi, const int *n_epi, const void *const *jw,
                  const int *n_epj, const void *const *sw, const int *n_spj, bool index) {
    SPH_TAG_LOCK(tag);
    TagState *ts = nullptr;
    Layout L;
    const size_t s_j = index ? sizeof(int) : sizeof(sph_epj_grav), s_s = index ? sizeof(int) : sizeof(sph_spj_monopole);
    JSrc<sph_epj_grav> rj{};
    JSrc<sph_spj_monopole> rs{};
    if (index) SPH_TRY((resident_src<sph_epj_grav, sph_spj_monopole>(3, n_walk, n_epj, n_spj, &rj, &rs)));
    SPH_TRY((stage<sph_epi_grav, sph_result_grav>(tag, 3, n_walk, epi, n_epi, jw, s_j, n_epj, sw, s_s, n_spj, index,
                                                  &ts, &L)));
    // from here on the dispatch runs to finish_dispatch, which waits for a device gather
    if (n_walk > 0) {
        JSrc<sph_epj_grav> js{(const sph_epj_grav *)(ts->d_in + L.o_epj), nullptr, 0, nullptr};
        JSrc<sph_spj_monopole> ss{(const sph_spj_monopole *)(ts->d_in + L.o_spj), nullptr, 0, nullptr};
        if (index) {
            js = JSrc<sph_epj_grav>{rj.base, (const int *)(ts->d_in + L.o_epj), rj.n, ts->d_err};
            ss = JSrc<sph_spj_monopole>{rs.base, (const int *)(ts->d_in + L.o_spj), rs.n, ts->d_err};
        }
        const sph_epi_grav *ei = (const sph_epi_grav *)ts->d_in;
        sph_result_grav *res = (sph_result_grav *)ts->d_out;
        if (g_batch_prec.load() == SPH_PREC_MIXED) batch32_grav(n_walk, ts->stream, ts->d_meta, ei, js, ss, res);
        else k_walk_grav<<<n_walk, WT, 0, ts->stream>>>(ts->d_meta, ei, js, ss, res);
    }
    return finish_dispatch(ts);
}

auto launch_dens = [](TagState *ts, const sph_epi_dens *ei, JSrc<sph_epj_dens> js, sph_result_dens *res, bool mixed) {
    const int n_walk = ts->pending_walks;
    if (mixed) batch32_dens(n_walk, ts->stream, ts->d_meta, ei, js, res);
    else k_walk_dens<<<n_walk, WT, 0, ts->stream>>>(ts->d_meta, ei, js, res);
};
auto launch_drvt = [](TagState *ts, const sph_epi_drvt *ei, JSrc<sph_epj_drvt> js, sph_result_drvt *res, bool mixed) {
    const int n_walk = ts->pending_walks;
    if (mixed) batch32_drvt(n_walk, ts->stream, ts->d_meta, ei, js, res);
    else k_walk_drvt<<<n_walk, WT, 0, ts->stream>>>(ts->d_meta, ei, js, res);
};
auto launch_hydro = [](TagState *ts, const sph_epi_hydro *ei, JSrc<sph_epj_hydro> js, sph_result_hydro *res,
                       bool mixed) {
    const int n_walk = ts->pending_walks;
    if (mixed) batch32_hydro(n_walk, ts->stream, ts->d_meta, ei, js, res);
    else k_walk_hydro<<<n_walk, WT, 0, ts->stream>>>(ts->d_meta, ei, js, res);
};

}  // namespace

extern "C" {

const char *sph_batch_last_error(void) { return g_batch_err.c_str(); }

int sph_batch_set_staging(int mode) {
    if (mode != SPH_BATCH_STAGING_AUTO && mode != SPH_BATCH_STAGING_HOST && mode != SPH_BATCH_STAGING_DEVICE)
        return batch_fail(SPH_ERR_ARG, "staging must be SPH_BATCH_STAGING_AUTO, _HOST or _DEVICE");
    g_batch_staging.store(mode);
    return SPH_OK;
}

int sph_batch_set_precision(int precision) {
    if (precision != SPH_PREC_FP64 && precision != SPH_PREC_MIXED)
        return batch_fail(SPH_ERR_ARG, "precision must be SPH_PREC_FP64 or SPH_PREC_MIXED");
    g_batch_prec.store(precision);
    return SPH_OK;
}

// ---- payload form (calcForceAllAndWriteBackMultiWalk)

int sph_dispatch_dens(int tag, int n_walk, const sph_epi_dens **epi, const int *n_epi, const sph_epj_dens **epj,
                      const int *n_epj) {
    return dispatch_walks<sph_epi_dens, sph_epj_dens, sph_result_dens>(tag, 0, n_walk, epi, n_epi,
                                                                       (const void *const *)epj, n_epj, false,
                                                                       launch_dens);
}

int sph_dispatch_drvt(int tag, int n_walk, const sph_epi_drvt **epi, const int *n_epi, const sph_epj_drvt **epj,
                      const int *n_epj) {
    return dispatch_walks<sph_epi_drvt, sph_epj_drvt, sph_result_drvt>(tag, 1, n_walk, epi, n_epi,
                                                                       (const void *const *)epj, n_epj, false,
                                                                       launch_drvt);
}

int sph_dispatch_hydro(int tag, int n_walk, const sph_epi_hydro **epi, const int *n_epi, const sph_epj_hydro **epj,
                       const int *n_epj) {
    return dispatch_walks<sph_epi_hydro, sph_epj_hydro, sph_result_hydro>(tag, 2, n_walk, epi, n_epi,
                                                                          (const void *const *)epj, n_epj, false,
                                                                          launch_hydro);
}

int sph_dispatch_grav(int tag, int n_walk, const sph_epi_grav **epi, const int *n_epi, const sph_epj_grav **epj,
                      const int *n_epj, const sph_spj_monopole **spj, const int *n_spj) {
    return dispatch_grav(tag, n_walk, epi, n_epi, (const void *const *)epj, n_epj, (const void *const *)spj, n_spj,
                         false);
}

// ---- index form (calcForceAllAndWriteBackMultiWalkIndex)

int sph_dispatch_index_dens(int tag, int n_walk, const sph_epi_dens **epi, const int *n_epi, const int **id_epj,
                            const int *n_epj, const sph_epj_dens *epj, int n_epj_tot, int send_flag) {
    if (send_flag) SPH_TRY(send_resident(0, epj, n_epj_tot, sizeof(sph_epj_dens), nullptr, 0, 1));
    if (n_walk == 0 && send_flag) return SPH_OK;
    return dispatch_walks<sph_epi_dens, sph_epj_dens, sph_result_dens>(tag, 0, n_walk, epi, n_epi,
                                                                       (const void *const *)id_epj, n_epj, true,
                                                                       launch_dens);
}

int sph_dispatch_index_drvt(int tag, int n_walk, const sph_epi_drvt **epi, const int *n_epi, const int **id_epj,
                            const int *n_epj, const sph_epj_drvt *epj, int n_epj_tot, int send_flag) {
    if (send_flag) SPH_TRY(send_resident(1, epj, n_epj_tot, sizeof(sph_epj_drvt), nullptr, 0, 1));
    if (n_walk == 0 && send_flag) return SPH_OK;
    return dispatch_walks<sph_epi_drvt, sph_epj_drvt, sph_result_drvt>(tag, 1, n_walk, epi, n_epi,
                                                                       (const void *const *)id_epj, n_epj, true,
                                                                       launch_drvt);
}

int sph_dispatch_index_hydro(int tag, int n_walk, const sph_epi_hydro **epi, const int *n_epi, const int **id_epj,
                             const int *n_epj, const sph_epj_hydro *epj, int n_epj_tot, int send_flag) {
    if (send_flag) SPH_TRY(send_resident(2, epj, n_epj_tot, sizeof(sph_epj_hydro), nullptr, 0, 1));
    if (n_walk == 0 && send_flag) return SPH_OK;
    return dispatch_walks<sph_epi_hydro, sph_epj_hydro, sph_result_hydro>(tag, 2, n_walk, epi, n_epi,
                                                                          (const void *const *)id_epj, n_epj, true,
                                                                          launch_hydro);
}

int sph_dispatch_index_grav(int tag, int n_walk, const sph_epi_grav **epi, const int *n_epi, const int **id_epj,
                            const int *n_epj, const int **id_spj, const int *n_spj, const sph_epj_grav *epj,
                            int n_epj_tot, const sph_spj_monopole *spj, int n_spj_tot, int send_flag) {
    if (send_flag)
        SPH_TRY(send_resident(3, epj, n_epj_tot, sizeof(sph_epj_grav), spj, n_spj_tot, sizeof(sph_spj_monopole)));
    if (n_walk == 0 && send_flag) return SPH_OK;
    return dispatch_grav(tag, n_walk, epi, n_epi, (const void *const *)id_epj, n_epj, (const void *const *)id_spj,
                         n_spj, true);
}

int sph_retrieve_dens(int tag, int n_walk, const int *n_epi, sph_result_dens **result) {
    return retrieve<sph_result_dens>(tag, 0, n_walk, n_epi, result);
}

int sph_retrieve_drvt(int tag, int n_walk, const int *n_epi, sph_result_drvt **result) {
    return retrieve<sph_result_drvt>(tag, 1, n_walk, n_epi, result);
}

int sph_retrieve_hydro(int tag, int n_walk, const int *n_epi, sph_result_hydro **result) {
    return retrieve<sph_result_hydro>(tag, 2, n_walk, n_epi, result);
}

int sph_retrieve_grav(int tag, int n_walk, const int *n_epi, sph_result_grav **result) {
    return retrieve<sph_result_grav>(tag, 3, n_walk, n_epi, result);
}

}  // extern "C"
