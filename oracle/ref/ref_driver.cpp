// Driver that runs the reference's own physics code (unmodified headers from
// the reference's src/ directory) on binary inputs and writes binary outputs.
// It is the reference leg of the oracle: test infrastructure that produces
// golden vectors and pins the C restatement in oracle/sph_oracle.c.  It is
// never linked into, or called by, the product library.
//
// Header order follows main.cpp:9-17; FLAG_GI is defined before force.h the
// way GI.h:4-5 does it for main.cpp.
//
// Usage: ref_driver MODE INPUT OUTPUT   (binary, native little-endian)
//   kernel   : n, {dx,dy,dz,h}[n]                    -> {W, gx, gy, gz}[n]
//   dens|drvt|hydro|grav : walk file (see read_walks) -> RESULT[sum n_i]
//   eos_file : len, path, kind, n, {rho,u}[n]        -> {P, cs}[n]
//   eos_static : which, n, {rho,u}[n]                -> {P, cs}[n]  (cwd = reference root)
//   eos_mode2 : len, path, kind, grid, n, {rho,s,u}[n]
//               -> {InternalEnergy(rho, s, grid), Temperature(rho, u), Entropy(rho, u)}[n]
//   balsara  : n, {div_v, rx, ry, rz, grad_smth, snds, smth}[n] -> {Bal, grad_smth, div_v}[n]
//   integ    : n, dt, damping, record[n]             -> record_out[n]
//   dtglobal : n, {dt, ax, ay, az, gx, gy, gz}[n]    -> dt
//   tillotson : par[10], len, path, n, {rho,u}[n]     -> {P_co, P_ex}[n]  (cwd = reference root)
#include "ps_shim.hpp"

#include "param.h"
#include "mathfunc.h"
#include "kernel.h"
#include "EoS.h"
#include "class.h"
#define SELF_GRAVITY
#define FLAG_GI
#include "force.h"
#include "integral.h"

// The analytic Tillotson branches P_co / P_ex (EoS.h:91-103) are private members of the
// reference's class and never called by it.  The golden generator reads them without touching
// the reference's headers: an explicit instantiation may name a private member ([temp.explicit]),
// and the friend function it defines hands out the member pointer.
namespace tillotson_access {
using Till = EoS::Tillotson<PS::F64>;
typedef PS::F64 (Till::*branch_fn)(PS::F64, PS::F64) const;
template <class Tag, branch_fn M>
struct Expose {
    friend branch_fn member(Tag) { return M; }
};
struct Pco {
    friend branch_fn member(Pco);
};
struct Pex {
    friend branch_fn member(Pex);
};
template struct Expose<Pco, &Till::P_co>;
template struct Expose<Pex, &Till::P_ex>;
}  // namespace tillotson_access

namespace {

struct Reader {
    FILE *fp;
    explicit Reader(const char *path) : fp(std::fopen(path, "rb")) {
        if (!fp) { std::fprintf(stderr, "cannot open %s\n", path); std::exit(2); }
    }
    ~Reader() { if (fp) std::fclose(fp); }
    template <class T> T get() {
        T v;
        if (std::fread(&v, sizeof(T), 1, fp) != 1) { std::fprintf(stderr, "short read\n"); std::exit(2); }
        return v;
    }
    template <class T> void get(T *dst, size_t n) {
        if (n && std::fread(dst, sizeof(T), n, fp) != n) { std::fprintf(stderr, "short read\n"); std::exit(2); }
    }
};

struct Writer {
    FILE *fp;
    explicit Writer(const char *path) : fp(std::fopen(path, "wb")) {
        if (!fp) { std::fprintf(stderr, "cannot open %s\n", path); std::exit(2); }
    }
    ~Writer() { if (fp) std::fclose(fp); }
    template <class T> void put(const T *src, size_t n) { if (n) std::fwrite(src, sizeof(T), n, fp); }
    template <class T> void put(const T v) { std::fwrite(&v, sizeof(T), 1, fp); }
};

// Walk file: int32 n_walk; per walk int32 n_i, n_j, n_s; EPI[n_i]; EPJ[n_j]; SPJ[n_s].
// The reference structs are read as raw bytes: every member is F64 or S64.
template <class EPI, class EPJ, class RES, class F>
void run_walks(Reader &in, Writer &out, F functor) {
    const int n_walk = in.get<int32_t>();
    for (int w = 0; w < n_walk; ++w) {
        const int n_i = in.get<int32_t>();
        const int n_j = in.get<int32_t>();
        const int n_s = in.get<int32_t>();
        std::vector<EPI> epi(n_i);
        std::vector<EPJ> epj(n_j);
        std::vector<PS::SPJMonopole> spj(n_s);
        in.get(epi.data(), n_i);
        in.get(epj.data(), n_j);
        in.get(spj.data(), n_s);
        std::vector<RES> res(n_i);
        for (auto &r : res) r.clear();  // FDPS clears RESULT before the functor
        functor(epi, epj, spj, res);
        out.put(res.data(), res.size());
    }
}

}  // namespace

static_assert(sizeof(STD::EPI::Dens) == 48, "EPI::Dens layout");
static_assert(sizeof(STD::EPJ::Dens) == 40, "EPJ::Dens layout");
static_assert(sizeof(STD::RESULT::Dens) == 16, "RESULT::Dens layout");
static_assert(sizeof(STD::EPI::Drvt) == 64, "EPI::Drvt layout");
static_assert(sizeof(STD::EPJ::Drvt) == 64, "EPJ::Drvt layout");
static_assert(sizeof(STD::RESULT::Drvt) == 40, "RESULT::Drvt layout");
static_assert(sizeof(STD::EPI::Hydro) == 112, "EPI::Hydro layout");
static_assert(sizeof(STD::EPJ::Hydro) == 120, "EPJ::Hydro layout");
static_assert(sizeof(STD::RESULT::Hydro) == 40, "RESULT::Hydro layout");
static_assert(sizeof(STD::EPI::Grav) == 40, "EPI::Grav layout");
static_assert(sizeof(STD::EPJ::Grav) == 40, "EPJ::Grav layout");
static_assert(sizeof(STD::RESULT::Grav) == 40, "RESULT::Grav layout");
static_assert(sizeof(PS::SPJMonopole) == 32, "SPJMonopole layout");

int main(int argc, char **argv) {
    if (argc != 4) {
        std::fprintf(stderr, "usage: %s MODE INPUT OUTPUT\n", argv[0]);
        return 2;
    }
    const std::string mode = argv[1];
    Reader in(argv[2]);
    Writer out(argv[3]);

    if (mode == "kernel") {
        kernel_t k;
        const int n = in.get<int32_t>();
        for (int i = 0; i < n; ++i) {
            double rec[4];
            in.get(rec, 4);
            const PS::F64vec dr(rec[0], rec[1], rec[2]);
            const PS::F64vec g = k.gradW(dr, rec[3]);
            const double o[4] = {k.W(dr, rec[3]), g.x, g.y, g.z};
            out.put(o, 4);
        }
    } else if (mode == "dens") {
        run_walks<STD::EPI::Dens, STD::EPJ::Dens, STD::RESULT::Dens>(
            in, out, [](auto &epi, auto &epj, auto &, auto &res) {
                STD::CalcDensity f;
                f(epi.data(), (PS::S32)epi.size(), epj.data(), (PS::S32)epj.size(), res.data());
            });
    } else if (mode == "drvt") {
        run_walks<STD::EPI::Drvt, STD::EPJ::Drvt, STD::RESULT::Drvt>(
            in, out, [](auto &epi, auto &epj, auto &, auto &res) {
                STD::CalcDerivative f;
                f(epi.data(), (PS::S32)epi.size(), epj.data(), (PS::S32)epj.size(), res.data());
            });
    } else if (mode == "hydro") {
        run_walks<STD::EPI::Hydro, STD::EPJ::Hydro, STD::RESULT::Hydro>(
            in, out, [](auto &epi, auto &epj, auto &, auto &res) {
                STD::CalcHydroForce f;
                f(epi.data(), (PS::S32)epi.size(), epj.data(), (PS::S32)epj.size(), res.data());
            });
    } else if (mode == "grav") {
        // FDPS calls the EPJ functor and then the SPJ functor into the same result (main.cpp:100-101).
        run_walks<STD::EPI::Grav, STD::EPJ::Grav, STD::RESULT::Grav>(
            in, out, [](auto &epi, auto &epj, auto &spj, auto &res) {
                STD::CalcGravityForce<STD::EPJ::Grav> fe;
                STD::CalcGravityForce<PS::SPJMonopole> fs;
                fe(epi.data(), (PS::S32)epi.size(), epj.data(), (PS::S32)epj.size(), res.data());
                fs(epi.data(), (PS::S32)epi.size(), spj.data(), (PS::S32)spj.size(), res.data());
            });
    } else if (mode == "eos_file") {
        const int len = in.get<int32_t>();
        std::string path(len, '\0');
        in.get(&path[0], len);
        const int kind = in.get<int32_t>();  // 0 = ANEOS class, 1 = Tillotson class (both table-backed)
        const int n = in.get<int32_t>();
        const EoS::EoS_t<PS::F64> *eos = nullptr;
        EoS::ANEOS<PS::F64> *an = nullptr;
        EoS::Tillotson<PS::F64> *ti = nullptr;
        if (kind == 0) {
            an = new EoS::ANEOS<PS::F64>(path);
            eos = an;
        } else {
            // Granite parameters as at EoS.h:446; Pressure/SoundSpeed read only the table.
            ti = new EoS::Tillotson<PS::F64>(2680.0, 16.0e+6, 3.5e+6, 18.00e+6, 18.0e+9, 18.0e+9, 0.5, 1.3, 5.0,
                                             5.0, path);
            eos = ti;
        }
        for (int i = 0; i < n; ++i) {
            double ru[2];
            in.get(ru, 2);
            const double o[2] = {eos->Pressure(ru[0], ru[1]), eos->SoundSpeed(ru[0], ru[1])};
            out.put(o, 2);
        }
        delete an;
        delete ti;
    } else if (mode == "eos_mode2") {
        // The mode-2 EoS surface (EoS.h:249-260, 402-413).  InternalEnergy
        // ignores its grid_size argument and passes 120 (EoS.h:250-251).
        const int len = in.get<int32_t>();
        std::string path(len, '\0');
        in.get(&path[0], len);
        const int kind = in.get<int32_t>();
        const int grid = in.get<int32_t>();
        const int n = in.get<int32_t>();
        const EoS::EoS_t<PS::F64> *eos = nullptr;
        EoS::ANEOS<PS::F64> *an = nullptr;
        EoS::Tillotson<PS::F64> *ti = nullptr;
        if (kind == 0) {
            an = new EoS::ANEOS<PS::F64>(path);
            eos = an;
        } else {
            ti = new EoS::Tillotson<PS::F64>(2680.0, 16.0e+6, 3.5e+6, 18.00e+6, 18.0e+9, 18.0e+9, 0.5, 1.3, 5.0,
                                             5.0, path);
            eos = ti;
        }
        for (int i = 0; i < n; ++i) {
            double rsu[3];
            in.get(rsu, 3);
            const double o[3] = {eos->InternalEnergy(rsu[0], rsu[1], grid), eos->Temperature(rsu[0], rsu[2]),
                                 eos->Entropy(rsu[0], rsu[2])};
            out.put(o, 3);
        }
        delete an;
        delete ti;
    } else if (mode == "eos_static") {
        const int which = in.get<int32_t>();  // 0 Granite (Tillotson), 1 Iron (ANEOS), 2 AGranite (ANEOS)
        const int n = in.get<int32_t>();
        const EoS::EoS_t<PS::F64> *eos = which == 0 ? (const EoS::EoS_t<PS::F64> *)&Granite
                                         : which == 1 ? (const EoS::EoS_t<PS::F64> *)&Iron
                                                      : (const EoS::EoS_t<PS::F64> *)&AGranite;
        for (int i = 0; i < n; ++i) {
            double ru[2];
            in.get(ru, 2);
            const double o[2] = {eos->Pressure(ru[0], ru[1]), eos->SoundSpeed(ru[0], ru[1])};
            out.put(o, 2);
        }
    } else if (mode == "balsara") {
        const int n = in.get<int32_t>();
        for (int i = 0; i < n; ++i) {
            double rec[7];
            in.get(rec, 7);
            STD::RESULT::Drvt r;
            r.div_v = rec[0];
            r.rot_v = PS::F64vec(rec[1], rec[2], rec[3]);
            r.grad_smth = rec[4];
            STD::RealPtcl p;
            p.snds = rec[5];
            p.smth = rec[6];
            p.copyFromForce(r);
            const double o[3] = {p.Bal, p.grad_smth, p.div_v};
            out.put(o, 3);
        }
    } else if (mode == "integ") {
        // record in : pos3 vel3 acc3 grav3 eng eng_dot | acc_new3 grav_new3 eng_dot_new  (21 doubles)
        // record out: pos3 vel3 vel_half3 eng eng_half (after kick-drift-predict) | vel3 eng (after final kick + damping)
        const int n = in.get<int32_t>();
        const double dt = in.get<double>();
        const double damping = in.get<double>();
        for (int i = 0; i < n; ++i) {
            double r[21];
            in.get(r, 21);
            STD::RealPtcl p;
            p.pos = PS::F64vec(r[0], r[1], r[2]);
            p.vel = PS::F64vec(r[3], r[4], r[5]);
            p.acc = PS::F64vec(r[6], r[7], r[8]);
            p.grav = PS::F64vec(r[9], r[10], r[11]);
            p.eng = r[12];
            p.eng_dot = r[13];
            p.initialKick(dt);
            p.fullDrift(dt);
            p.predict(dt);
            const double o1[11] = {p.pos.x, p.pos.y, p.pos.z, p.vel.x, p.vel.y, p.vel.z,
                                   p.vel_half.x, p.vel_half.y, p.vel_half.z, p.eng, p.eng_half};
            out.put(o1, 11);
            p.acc = PS::F64vec(r[14], r[15], r[16]);
            p.grav = PS::F64vec(r[17], r[18], r[19]);
            p.eng_dot = r[20];
            p.finalKick(dt);
            p.dampMotion(damping);
            const double o2[4] = {p.vel.x, p.vel.y, p.vel.z, p.eng};
            out.put(o2, 4);
        }
    } else if (mode == "dtglobal") {
        const int n = in.get<int32_t>();
        PS::ParticleSystem<STD::RealPtcl> sys;
        sys.setNumberOfParticleLocal(n);
        for (int i = 0; i < n; ++i) {
            double r[7];
            in.get(r, 7);
            sys[i].dt = r[0];
            sys[i].acc = PS::F64vec(r[1], r[2], r[3]);
            sys[i].grav = PS::F64vec(r[4], r[5], r[6]);
        }
        out.put(getTimeStepGlobal<STD::RealPtcl>(sys));
    } else if (mode == "tillotson") {
        // P_co and P_ex of a Tillotson object built with the given parameters (constructor order
        // rho0 u0 uiv ucv A B a b alpha beta, EoS.h:105-107); the table file the constructor also
        // reads does not enter them.
        double par[10];
        in.get(par, 10);
        const int len = in.get<int32_t>();
        std::string path(len, '\0');
        in.get(&path[0], len);
        const int n = in.get<int32_t>();
        const tillotson_access::Till t(par[0], par[1], par[2], par[3], par[4], par[5], par[6], par[7], par[8],
                                       par[9], path);
        const tillotson_access::branch_fn pco = member(tillotson_access::Pco());
        const tillotson_access::branch_fn pex = member(tillotson_access::Pex());
        for (int i = 0; i < n; ++i) {
            double ru[2];
            in.get(ru, 2);
            const double o[2] = {(t.*pco)(ru[0], ru[1]), (t.*pex)(ru[0], ru[1])};
            out.put(o, 2);
        }
    } else {
        std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
        return 2;
    }
    return 0;
}
