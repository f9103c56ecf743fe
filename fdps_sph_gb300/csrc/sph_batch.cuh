// Shared by the batch entry points (sph_batch.cu) and their mixed-precision kernels
// (sph_batch32.cu).
#pragma once

#include "sph_physics.cuh"

namespace sph {

// The j entries of one dispatch's walks, entry k of the walk starting at offset jo being
// src[jo + k].  Payload form (calcForceAllAndWriteBackMultiWalk): idx == nullptr, the entries are
// the staged payloads themselves, base[k].  Index form (calcForceAllAndWriteBackMultiWalkIndex):
// the staged entries are indices into an array sent once per pass, base[idx[k]]; an index outside
// [0, n) sets bit 0 of *err and reads entry 0 instead (the host refuses index walks when the sent
// array is empty), so a bad index cannot read past the array.
template <class T>
struct JSrc {
    const T *base;
    const int *idx;
    int64_t n;
    int *err;
    __device__ __forceinline__ const T &operator[](int64_t k) const {
        if (!idx) return base[k];
        int j = idx[k];
        if ((unsigned long long)(long long)j >= (unsigned long long)n) {
            atomicOr(err, 1);
            j = 0;
        }
        return base[j];
    }
};

// the mixed-precision functor kernels (sph_batch32.cu): one block per walk on the tag's stream
void batch32_dens(int n_walk, cudaStream_t st, const int64_t *meta, const sph_epi_dens *epi, JSrc<sph_epj_dens> epj,
                  sph_result_dens *res);
void batch32_drvt(int n_walk, cudaStream_t st, const int64_t *meta, const sph_epi_drvt *epi, JSrc<sph_epj_drvt> epj,
                  sph_result_drvt *res);
void batch32_hydro(int n_walk, cudaStream_t st, const int64_t *meta, const sph_epi_hydro *epi,
                   JSrc<sph_epj_hydro> epj, sph_result_hydro *res);
void batch32_grav(int n_walk, cudaStream_t st, const int64_t *meta, const sph_epi_grav *epi, JSrc<sph_epj_grav> epj,
                  JSrc<sph_spj_monopole> spj, sph_result_grav *res);

}  // namespace sph
