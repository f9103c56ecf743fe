// fdps_sph_gb300.hpp -- C++ host surface over the C ABI of libsph_gb300.so,
// shaped like the reference's own interface so FDPS_SPH host code can switch
// with minimal edits.
//
//  * CalcDensity / CalcDerivative / CalcHydroForce / CalcGravityForce: the
//    functor classes of force.h:6-172 with the same operator() signatures
//    (const EPI*, S32, const EPJ*, S32, RESULT*).  They run the reference
//    functor on the GPU for one i-group.  Any EPI / EPJ / RESULT type whose
//    layout is the reference's (class.h:34-454) is accepted; the layout is
//    checked at compile time.  The reference functors cannot fail; these
//    throw std::runtime_error when the GPU call fails (host side only).
//  * Dispatch* / Retrieve*: the callbacks calcForceAllAndWriteBackMultiWalk
//    takes, forwarding to sph_dispatch_* / sph_retrieve_*; DispatchIndex*:
//    the dispatch callbacks of calcForceAllAndWriteBackMultiWalkIndex (the
//    pass's EPJ / SPJ arrays sent once, walks as int32 indices), forwarding to
//    sph_dispatch_index_*, retrieved with the same Retrieve*.
//  * Simulation: RAII owner of a device-resident context (sph_ctx) running
//    the step of main.cpp:125-173 on the GPU.
#pragma once

#include <atomic>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "sph_gb300.h"

namespace sph_gb300 {

namespace detail {
inline void check_batch(int rc, const char *what) {
    if (rc != SPH_OK) throw std::runtime_error(std::string(what) + ": " + sph_batch_last_error());
}
// FDPS calls functors from several OpenMP threads at once.  Each calling thread
// takes a tag of its own (8 .. 63, round robin; 0 .. 7 stay free for a host's
// own MultiWalk dispatch / retrieve), so the threads' walks overlap on the GPU,
// one stream per tag.  A wrapper call holds its tag's lock across its dispatch
// / retrieve pair, which matters only when more than 56 threads share tags.
inline int thread_tag() {
    static std::atomic<int> next{0};
    thread_local const int tag = 8 + next.fetch_add(1) % 56;
    return tag;
}
inline std::mutex &tag_lock(int tag) {
    static std::mutex m[64];
    return m[tag];
}
template <class T, class C>
constexpr bool same_layout() {
    return sizeof(T) == sizeof(C) && alignof(T) <= alignof(C) + 8;
}
}  // namespace detail

// ---- functors with the reference signatures (force.h) ----------------------

struct CalcDensity {   // force.h:6-24
    template <class EPI, class EPJ, class RESULT>
    void operator()(const EPI *ep_i, int n_i, const EPJ *ep_j, int n_j, RESULT *dens) const {
        static_assert(detail::same_layout<EPI, sph_epi_dens>(), "EPI::Dens layout (class.h:233-258)");
        static_assert(detail::same_layout<EPJ, sph_epj_dens>(), "EPJ::Dens layout (class.h:342-365)");
        static_assert(detail::same_layout<RESULT, sph_result_dens>(), "RESULT::Dens layout (class.h:36-44)");
        const sph_epi_dens *pi = reinterpret_cast<const sph_epi_dens *>(ep_i);
        const sph_epj_dens *pj = reinterpret_cast<const sph_epj_dens *>(ep_j);
        sph_result_dens *out = reinterpret_cast<sph_result_dens *>(dens);
        const int tag = detail::thread_tag();
        std::lock_guard<std::mutex> lk(detail::tag_lock(tag));
        detail::check_batch(sph_dispatch_dens(tag, 1, &pi, &n_i, &pj, &n_j), "CalcDensity");
        detail::check_batch(sph_retrieve_dens(tag, 1, &n_i, &out), "CalcDensity");
    }
};

struct CalcDerivative {   // force.h:86-107
    template <class EPI, class EPJ, class RESULT>
    void operator()(const EPI *ep_i, int n_i, const EPJ *ep_j, int n_j, RESULT *drvt) const {
        static_assert(detail::same_layout<EPI, sph_epi_drvt>(), "EPI::Drvt layout (class.h:260-281)");
        static_assert(detail::same_layout<EPJ, sph_epj_drvt>(), "EPJ::Drvt layout (class.h:367-392)");
        static_assert(detail::same_layout<RESULT, sph_result_drvt>(), "RESULT::Drvt layout (class.h:47-58)");
        const sph_epi_drvt *pi = reinterpret_cast<const sph_epi_drvt *>(ep_i);
        const sph_epj_drvt *pj = reinterpret_cast<const sph_epj_drvt *>(ep_j);
        sph_result_drvt *out = reinterpret_cast<sph_result_drvt *>(drvt);
        const int tag = detail::thread_tag();
        std::lock_guard<std::mutex> lk(detail::tag_lock(tag));
        detail::check_batch(sph_dispatch_drvt(tag, 1, &pi, &n_i, &pj, &n_j), "CalcDerivative");
        detail::check_batch(sph_retrieve_drvt(tag, 1, &n_i, &out), "CalcDerivative");
    }
};

struct CalcHydroForce {   // force.h:109-148
    template <class EPI, class EPJ, class RESULT>
    void operator()(const EPI *ep_i, int n_i, const EPJ *ep_j, int n_j, RESULT *hydro) const {
        static_assert(detail::same_layout<EPI, sph_epi_hydro>(), "EPI::Hydro layout (class.h:283-315)");
        static_assert(detail::same_layout<EPJ, sph_epj_hydro>(), "EPJ::Hydro layout (class.h:394-432)");
        static_assert(detail::same_layout<RESULT, sph_result_hydro>(), "RESULT::Hydro layout (class.h:61-72)");
        const sph_epi_hydro *pi = reinterpret_cast<const sph_epi_hydro *>(ep_i);
        const sph_epj_hydro *pj = reinterpret_cast<const sph_epj_hydro *>(ep_j);
        sph_result_hydro *out = reinterpret_cast<sph_result_hydro *>(hydro);
        const int tag = detail::thread_tag();
        std::lock_guard<std::mutex> lk(detail::tag_lock(tag));
        detail::check_batch(sph_dispatch_hydro(tag, 1, &pi, &n_i, &pj, &n_j), "CalcHydroForce");
        detail::check_batch(sph_retrieve_hydro(tag, 1, &n_i, &out), "CalcHydroForce");
    }
};

// force.h:150-172; TPtclJ is EPJ::Grav or PS::SPJMonopole.  The reference
// calls the EPJ functor and then the SPJ functor into the same RESULT; the
// GPU call covers one list, so a result already holding the EPJ sum is
// continued by passing it back in (the kernel accumulates from RESULT::clear,
// the sum is completed here).
template <class TPtclJ>
struct CalcGravityForce {
    template <class EPI, class RESULT>
    void operator()(const EPI *ep_i, int n_i, const TPtclJ *ep_j, int n_j, RESULT *grav) const {
        static_assert(detail::same_layout<EPI, sph_epi_grav>(), "EPI::Grav layout (class.h:317-338)");
        static_assert(detail::same_layout<RESULT, sph_result_grav>(), "RESULT::Grav layout (class.h:75-86)");
        static_assert(sizeof(TPtclJ) == sizeof(sph_epj_grav) || sizeof(TPtclJ) == sizeof(sph_spj_monopole),
                      "EPJ::Grav (class.h:434-453) or SPJMonopole");
        const sph_epi_grav *pi = reinterpret_cast<const sph_epi_grav *>(ep_i);
        std::vector<sph_result_grav> tmp(n_i > 0 ? n_i : 1);
        sph_result_grav *out = tmp.data();
        const int zero = 0;
        const int tag = detail::thread_tag();
        std::lock_guard<std::mutex> lk(detail::tag_lock(tag));
        if (sizeof(TPtclJ) == sizeof(sph_epj_grav)) {
            const sph_epj_grav *pj = reinterpret_cast<const sph_epj_grav *>(ep_j);
            const sph_spj_monopole *ps = nullptr;
            detail::check_batch(sph_dispatch_grav(tag, 1, &pi, &n_i, &pj, &n_j, &ps, &zero), "CalcGravityForce");
        } else {
            const sph_epj_grav *pj = nullptr;
            const sph_spj_monopole *ps = reinterpret_cast<const sph_spj_monopole *>(ep_j);
            detail::check_batch(sph_dispatch_grav(tag, 1, &pi, &n_i, &pj, &zero, &ps, &n_j), "CalcGravityForce");
        }
        detail::check_batch(sph_retrieve_grav(tag, 1, &n_i, &out), "CalcGravityForce");
        sph_result_grav *g = reinterpret_cast<sph_result_grav *>(grav);
        for (int i = 0; i < n_i; ++i) {   // acc -= ..., pot -= ... accumulate into the caller's result
            g[i].acc[0] += out[i].acc[0];
            g[i].acc[1] += out[i].acc[1];
            g[i].acc[2] += out[i].acc[2];
            g[i].pot += out[i].pot;
        }
    }
};

// ---- MultiWalk callbacks -----------------------------------------------------

template <class EPI, class EPJ>
int DispatchDens(int tag, int n_walk, const EPI **epi, const int *n_epi, const EPJ **epj, const int *n_epj) {
    static_assert(detail::same_layout<EPI, sph_epi_dens>() && detail::same_layout<EPJ, sph_epj_dens>(), "layout");
    return sph_dispatch_dens(tag, n_walk, reinterpret_cast<const sph_epi_dens **>(epi), n_epi,
                             reinterpret_cast<const sph_epj_dens **>(epj), n_epj);
}
template <class RESULT>
int RetrieveDens(int tag, int n_walk, const int *n_epi, RESULT **result) {
    return sph_retrieve_dens(tag, n_walk, n_epi, reinterpret_cast<sph_result_dens **>(result));
}
template <class EPI, class EPJ>
int DispatchDrvt(int tag, int n_walk, const EPI **epi, const int *n_epi, const EPJ **epj, const int *n_epj) {
    static_assert(detail::same_layout<EPI, sph_epi_drvt>() && detail::same_layout<EPJ, sph_epj_drvt>(), "layout");
    return sph_dispatch_drvt(tag, n_walk, reinterpret_cast<const sph_epi_drvt **>(epi), n_epi,
                             reinterpret_cast<const sph_epj_drvt **>(epj), n_epj);
}
template <class RESULT>
int RetrieveDrvt(int tag, int n_walk, const int *n_epi, RESULT **result) {
    return sph_retrieve_drvt(tag, n_walk, n_epi, reinterpret_cast<sph_result_drvt **>(result));
}
template <class EPI, class EPJ>
int DispatchHydro(int tag, int n_walk, const EPI **epi, const int *n_epi, const EPJ **epj, const int *n_epj) {
    static_assert(detail::same_layout<EPI, sph_epi_hydro>() && detail::same_layout<EPJ, sph_epj_hydro>(), "layout");
    return sph_dispatch_hydro(tag, n_walk, reinterpret_cast<const sph_epi_hydro **>(epi), n_epi,
                              reinterpret_cast<const sph_epj_hydro **>(epj), n_epj);
}
template <class RESULT>
int RetrieveHydro(int tag, int n_walk, const int *n_epi, RESULT **result) {
    return sph_retrieve_hydro(tag, n_walk, n_epi, reinterpret_cast<sph_result_hydro **>(result));
}
template <class EPI, class EPJ, class SPJ>
int DispatchGrav(int tag, int n_walk, const EPI **epi, const int *n_epi, const EPJ **epj, const int *n_epj,
                 const SPJ **spj, const int *n_spj) {
    static_assert(detail::same_layout<EPI, sph_epi_grav>() && detail::same_layout<EPJ, sph_epj_grav>() &&
                      detail::same_layout<SPJ, sph_spj_monopole>(), "layout");
    return sph_dispatch_grav(tag, n_walk, reinterpret_cast<const sph_epi_grav **>(epi), n_epi,
                             reinterpret_cast<const sph_epj_grav **>(epj), n_epj,
                             reinterpret_cast<const sph_spj_monopole **>(spj), n_spj);
}
template <class RESULT>
int RetrieveGrav(int tag, int n_walk, const int *n_epi, RESULT **result) {
    return sph_retrieve_grav(tag, n_walk, n_epi, reinterpret_cast<sph_result_grav **>(result));
}

// ---- MultiWalkIndex dispatch callbacks (retrieve: the Retrieve* above) ----------

template <class EPI, class EPJ>
int DispatchIndexDens(int tag, int n_walk, const EPI **epi, const int *n_epi, const int **id_epj, const int *n_epj,
                      const EPJ *epj, int n_epj_tot, bool send_flag) {
    static_assert(detail::same_layout<EPI, sph_epi_dens>() && detail::same_layout<EPJ, sph_epj_dens>(), "layout");
    return sph_dispatch_index_dens(tag, n_walk, reinterpret_cast<const sph_epi_dens **>(epi), n_epi, id_epj, n_epj,
                                   reinterpret_cast<const sph_epj_dens *>(epj), n_epj_tot, send_flag ? 1 : 0);
}
template <class EPI, class EPJ>
int DispatchIndexDrvt(int tag, int n_walk, const EPI **epi, const int *n_epi, const int **id_epj, const int *n_epj,
                      const EPJ *epj, int n_epj_tot, bool send_flag) {
    static_assert(detail::same_layout<EPI, sph_epi_drvt>() && detail::same_layout<EPJ, sph_epj_drvt>(), "layout");
    return sph_dispatch_index_drvt(tag, n_walk, reinterpret_cast<const sph_epi_drvt **>(epi), n_epi, id_epj, n_epj,
                                   reinterpret_cast<const sph_epj_drvt *>(epj), n_epj_tot, send_flag ? 1 : 0);
}
template <class EPI, class EPJ>
int DispatchIndexHydro(int tag, int n_walk, const EPI **epi, const int *n_epi, const int **id_epj, const int *n_epj,
                       const EPJ *epj, int n_epj_tot, bool send_flag) {
    static_assert(detail::same_layout<EPI, sph_epi_hydro>() && detail::same_layout<EPJ, sph_epj_hydro>(), "layout");
    return sph_dispatch_index_hydro(tag, n_walk, reinterpret_cast<const sph_epi_hydro **>(epi), n_epi, id_epj, n_epj,
                                    reinterpret_cast<const sph_epj_hydro *>(epj), n_epj_tot, send_flag ? 1 : 0);
}
template <class EPI, class EPJ, class SPJ>
int DispatchIndexGrav(int tag, int n_walk, const EPI **epi, const int *n_epi, const int **id_epj, const int *n_epj,
                      const int **id_spj, const int *n_spj, const EPJ *epj, int n_epj_tot, const SPJ *spj,
                      int n_spj_tot, bool send_flag) {
    static_assert(detail::same_layout<EPI, sph_epi_grav>() && detail::same_layout<EPJ, sph_epj_grav>() &&
                      detail::same_layout<SPJ, sph_spj_monopole>(), "layout");
    return sph_dispatch_index_grav(tag, n_walk, reinterpret_cast<const sph_epi_grav **>(epi), n_epi, id_epj, n_epj,
                                   id_spj, n_spj, reinterpret_cast<const sph_epj_grav *>(epj), n_epj_tot,
                                   reinterpret_cast<const sph_spj_monopole *>(spj), n_spj_tot, send_flag ? 1 : 0);
}

// ---- device-resident run -------------------------------------------------------

class Simulation {
public:
    explicit Simulation(const sph_config *cfg = nullptr) {
        const int rc = sph_ctx_create(cfg, &ctx_);
        if (rc != SPH_OK) throw std::runtime_error("sph_ctx_create failed (" + std::to_string(rc) + ")");
    }
    ~Simulation() { sph_ctx_destroy(ctx_); }
    Simulation(const Simulation &) = delete;
    Simulation &operator=(const Simulation &) = delete;

    void check(int rc) const {
        if (rc != SPH_OK) throw std::runtime_error(sph_last_error(ctx_));
    }
    void table(int material, const char *path) { check(sph_load_eos_table_file(ctx_, material, path)); }
    void tillotson(int material, const double par[10]) { check(sph_set_eos_tillotson(ctx_, material, par)); }
    // fields: field-major block (sph_field order), ld >= n
    void upload(int64_t n, const double *fields, int64_t ld, const int64_t *id, const int32_t *material,
                double time = 0.0, int flags = 0, double dt = 0.0) {
        check(sph_upload(ctx_, n, fields, ld, id, material, time, dt, flags));
    }
    void download(double *fields, int64_t ld, int64_t *id, int32_t *material) {
        check(sph_download(ctx_, fields, ld, id, material));
    }
    void prologue() { check(sph_prologue(ctx_)); }   // main.cpp:92-105
    void step(int n = 1) { check(sph_step(ctx_, n)); }   // main.cpp:125-173
    double time() const {
        double t = 0.0;
        sph_get_time(ctx_, &t, nullptr, nullptr);
        return t;
    }
    double dt() const {
        double d = 0.0;
        sph_get_time(ctx_, nullptr, &d, nullptr);
        return d;
    }
    sph_ctx *handle() const { return ctx_; }

private:
    sph_ctx *ctx_ = nullptr;
};

}  // namespace sph_gb300
