// Host program written the way FDPS_SPH's own code calls its functors
// (force.h), with payload types declared like class.h, but running on the
// GPU through include/fdps_sph_gb300.hpp.  Reads walks of the golden
// fixtures (binary, written by tests/test_gpu_cpp_host.py) and writes the
// results.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>

#include "fdps_sph_gb300.hpp"

namespace PS {
typedef double F64;
typedef int S32;
typedef long long S64;
struct F64vec {
    F64 x, y, z;
};
struct SPJMonopole {
    F64 mass;
    F64vec pos;
};
}  // namespace PS

namespace STD {
namespace RESULT {
struct Dens { PS::F64 dens, smth; };
struct Hydro { PS::F64vec acc; PS::F64 eng_dot, dt; };
struct Grav { PS::F64vec acc; PS::F64 pot, dt; };
}  // namespace RESULT
namespace EPI {
struct Dens { PS::F64vec pos; PS::F64 mass, smth; PS::S64 id; };
struct Hydro {
    PS::F64vec pos, vel;
    PS::F64 smth, dens, pres, snds, grad_smth, Bal, AVa;
    PS::S64 id;
};
struct Grav { PS::F64vec pos; PS::F64 eps2; PS::S64 id; };
}  // namespace EPI
namespace EPJ {
struct Dens { PS::F64 mass; PS::F64vec pos; PS::F64 smth; };
struct Hydro {
    PS::F64vec pos, vel;
    PS::F64 dens, mass, smth, pres, grad_smth, snds, Bal, AVa;
    PS::S64 id;
};
struct Grav { PS::F64vec pos; PS::F64 mass; PS::S64 id; };
}  // namespace EPJ
}  // namespace STD

template <class T>
static std::vector<T> read_vec(FILE *f) {
    int32_t n = 0;
    if (std::fread(&n, 4, 1, f) != 1) return {};
    std::vector<T> v(n);
    if (n && std::fread(v.data(), sizeof(T), n, f) != (size_t)n) v.clear();
    return v;
}

int main(int argc, char **argv) {
    if (argc != 3) return 2;
    FILE *in = std::fopen(argv[1], "rb");
    FILE *out = std::fopen(argv[2], "wb");
    if (!in || !out) return 2;
    // density: one walk
    auto di = read_vec<STD::EPI::Dens>(in);
    auto dj = read_vec<STD::EPJ::Dens>(in);
    std::vector<STD::RESULT::Dens> dr(di.size(), STD::RESULT::Dens{0, 0});
    sph_gb300::CalcDensity()(di.data(), (PS::S32)di.size(), dj.data(), (PS::S32)dj.size(), dr.data());
    std::fwrite(dr.data(), sizeof(dr[0]), dr.size(), out);
    // hydro: one walk
    auto hi = read_vec<STD::EPI::Hydro>(in);
    auto hj = read_vec<STD::EPJ::Hydro>(in);
    std::vector<STD::RESULT::Hydro> hr(hi.size());
    sph_gb300::CalcHydroForce()(hi.data(), (PS::S32)hi.size(), hj.data(), (PS::S32)hj.size(), hr.data());
    std::fwrite(hr.data(), sizeof(hr[0]), hr.size(), out);
    // gravity: EPJ functor then SPJ functor into the same result (main.cpp:100-101)
    auto gi = read_vec<STD::EPI::Grav>(in);
    auto gj = read_vec<STD::EPJ::Grav>(in);
    auto gs = read_vec<PS::SPJMonopole>(in);
    std::vector<STD::RESULT::Grav> gr(gi.size(), STD::RESULT::Grav{{0, 0, 0}, 0, 1.0e30});
    sph_gb300::CalcGravityForce<STD::EPJ::Grav>()(gi.data(), (PS::S32)gi.size(), gj.data(), (PS::S32)gj.size(),
                                                   gr.data());
    sph_gb300::CalcGravityForce<PS::SPJMonopole>()(gi.data(), (PS::S32)gi.size(), gs.data(), (PS::S32)gs.size(),
                                                    gr.data());
    std::fwrite(gr.data(), sizeof(gr[0]), gr.size(), out);
    // the density and hydro functors called from eight threads at once, as FDPS's OpenMP threads
    // call them: every thread's results equal the single-threaded ones bit for bit
    const int n_thr = 8, reps = 20;
    std::vector<std::vector<STD::RESULT::Dens>> tdr(n_thr, dr);
    std::vector<std::vector<STD::RESULT::Hydro>> thr_(n_thr, hr);
    std::vector<int> bad(n_thr, 0);
    std::vector<std::thread> pool;
    for (int t = 0; t < n_thr; ++t)
        pool.emplace_back([&, t]() {
            for (int r = 0; r < reps; ++r) {
                std::vector<STD::RESULT::Dens> a(di.size(), STD::RESULT::Dens{0, 0});
                sph_gb300::CalcDensity()(di.data(), (PS::S32)di.size(), dj.data(), (PS::S32)dj.size(), a.data());
                std::vector<STD::RESULT::Hydro> b(hi.size());
                sph_gb300::CalcHydroForce()(hi.data(), (PS::S32)hi.size(), hj.data(), (PS::S32)hj.size(), b.data());
                if (std::memcmp(a.data(), dr.data(), sizeof(a[0]) * a.size()) != 0 ||
                    std::memcmp(b.data(), hr.data(), sizeof(b[0]) * b.size()) != 0)
                    bad[t] = 1;
            }
        });
    for (auto &th : pool) th.join();
    int n_bad = 0;
    for (int t = 0; t < n_thr; ++t) n_bad += bad[t];
    std::fwrite(&n_bad, sizeof(n_bad), 1, out);
    // the same hydro walk through the MultiWalk callbacks, payload form and index form (the EPJ
    // array sent first, the walk as indices into it): both bit-identical to the functor's results
    int mw_bad = 0;
    {
        const STD::EPI::Hydro *ep[1] = {hi.data()};
        const STD::EPJ::Hydro *jp[1] = {hj.data()};
        int ni[1] = {(int)hi.size()}, nj[1] = {(int)hj.size()};
        std::vector<STD::RESULT::Hydro> r1(hi.size()), r2(hi.size());
        STD::RESULT::Hydro *rp1[1] = {r1.data()}, *rp2[1] = {r2.data()};
        if (sph_gb300::DispatchHydro(6, 1, ep, ni, jp, nj) != 0 || sph_gb300::RetrieveHydro(6, 1, ni, rp1) != 0)
            mw_bad |= 1;
        std::vector<int> idx(hj.size());
        for (size_t k = 0; k < idx.size(); ++k) idx[k] = (int)k;
        const int *ip[1] = {idx.data()};
        if (sph_gb300::DispatchIndexHydro(6, 0, ep, ni, ip, nj, hj.data(), (int)hj.size(), true) != 0 ||
            sph_gb300::DispatchIndexHydro(6, 1, ep, ni, ip, nj, hj.data(), (int)hj.size(), false) != 0 ||
            sph_gb300::RetrieveHydro(6, 1, ni, rp2) != 0)
            mw_bad |= 2;
        if (std::memcmp(r1.data(), hr.data(), sizeof(hr[0]) * hr.size()) != 0) mw_bad |= 4;
        if (std::memcmp(r2.data(), hr.data(), sizeof(hr[0]) * hr.size()) != 0) mw_bad |= 8;
    }
    std::fwrite(&mw_bad, sizeof(mw_bad), 1, out);
    std::fclose(in);
    std::fclose(out);
    return 0;
}
