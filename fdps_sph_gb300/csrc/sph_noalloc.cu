// Allocation-free Morton ordering: the key and sort stage of the octree
// build (sph_tree.cu) for callers that must not allocate device memory.
//
// Who needs this: a host that runs under a fixed device-memory budget (an
// embedding application that has handed the rest of the GPU to its own pool
// allocator, or a service that must not grow its footprint while it runs)
// cannot let a library call cudaMalloc / cudaFree, and a cudaFree also
// synchronises the device, which such a host may not allow in the middle of
// a step.  This entry point takes device pointers for its inputs and
// outputs and keeps its scratch in one file-scope device array, sized for at
// most SPH_NOALLOC_MAX_N particles.  That array exists on every GPU that
// loads the library, for the lifetime of the process, whether or not the
// entry point is used.
//
// The array is shared by every call on a device and keeps the last call's
// contents; each call rewrites all of it that it reads except the error
// word, which it clears first.  Two calls whose work overlaps on the GPU
// (different streams, no ordering between them) race on the array.  Called
// eagerly, a call ends by reading the error word back to the host, so it
// returns only after its work on `stream` has finished.  Called while
// `stream` is being captured into a CUDA graph, it only records its work (the
// memset, the launches and the device-to-device copies are all capturable)
// and returns at once: a replay reports no status.
#include <mutex>

#include "sph_internal.cuh"

namespace sph {

// the key and sort kernels of sph_tree.cu (declared in sph_internal.cuh) are launched from here unchanged

namespace {

constexpr int NA_MAX = SPH_NOALLOC_MAX_N;
constexpr int NA_TILE = RS_TILE;                  // radix-sort tile (k_rs_scatter)
constexpr int NA_NB = (NA_MAX + NA_TILE - 1) / NA_TILE;
constexpr int NA_BOX = 304;                       // blocks of k_bbox_partial
constexpr int NA_SCAN = 256;                      // blocks of the scan kernels

// byte offsets inside the scratch array (each 256-byte aligned)
constexpr size_t al(size_t b) { return (b + 255) & ~size_t(255); }
constexpr size_t OFF_BOX = 0;                                           // double [NA_BOX * 6]
constexpr size_t OFF_RB = OFF_BOX + al(sizeof(double) * NA_BOX * 6);    // double [8 + 22]
constexpr size_t OFF_K0 = OFF_RB + al(sizeof(double) * 32);             // uint64 [NA_MAX]
constexpr size_t OFF_K1 = OFF_K0 + al(sizeof(uint64_t) * NA_MAX);
constexpr size_t OFF_V0 = OFF_K1 + al(sizeof(uint64_t) * NA_MAX);       // uint32 [NA_MAX]
constexpr size_t OFF_V1 = OFF_V0 + al(sizeof(uint32_t) * NA_MAX);
constexpr size_t OFF_HIST = OFF_V1 + al(sizeof(uint32_t) * NA_MAX);     // uint32 [256 * NA_NB]
constexpr size_t OFF_HOFF = OFF_HIST + al(sizeof(uint32_t) * 256 * NA_NB);
constexpr size_t OFF_PART = OFF_HOFF + al(sizeof(uint32_t) * 256 * NA_NB);   // int [NA_SCAN + 1]
constexpr size_t OFF_ERR = OFF_PART + al(sizeof(int) * (NA_SCAN + 1));       // int
constexpr size_t NA_BYTES = OFF_ERR + 256;

}  // namespace
}  // namespace sph

// the scratch: about 3.2 MB for SPH_NOALLOC_MAX_N = 131072
static __device__ __align__(256) unsigned char g_noalloc_scratch[sph::NA_BYTES];

namespace {

std::mutex g_na_mu;
unsigned char *g_na_ptr[64] = {nullptr};   // device address of the scratch, per device

// once per device, with that device current: the device address of the array
int noalloc_setup(int dev, unsigned char **out) {
    std::lock_guard<std::mutex> lk(g_na_mu);
    if (dev < 0 || dev >= 64) return SPH_ERR_CUDA;
    if (!g_na_ptr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return SPH_ERR_CUDA;
        }
        g_na_ptr[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_na_ptr[dev];
    return SPH_OK;
}

// the array's address is known on this device (a capture may not make the first call: it looks
// the address up)
bool noalloc_ready(int dev) {
    std::lock_guard<std::mutex> lk(g_na_mu);
    return dev >= 0 && dev < 64 && g_na_ptr[dev] != nullptr;
}

}  // namespace

extern "C" int sph_morton_order_noalloc(const double *x, const double *y, const double *z, int64_t n,
                                        uint64_t *keys_out, int32_t *order_out, void *stream) {
    using namespace sph;
    if (!x || !y || !z || !keys_out || !order_out || n < 1) return SPH_ERR_ARG;
    if (n > NA_MAX) return SPH_ERR_CAPACITY;   // the scratch holds at most SPH_NOALLOC_MAX_N particles
    // An error an earlier call left pending on this thread is reported before any work is queued and left
    // in place for its owner, so the launch checks below see this call's launches only.
    if (cudaPeekAtLastError() != cudaSuccess) return SPH_ERR_CUDA;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return SPH_ERR_CUDA;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaStreamCaptureStatus capture = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &capture) != cudaSuccess) {
        cudaGetLastError();
        return SPH_ERR_CUDA;
    }
    const bool capturing = capture == cudaStreamCaptureStatusActive;
    if (capturing && !noalloc_ready(dev)) return SPH_ERR_STATE;   // nothing recorded
    unsigned char *base = nullptr;
    const int rc = noalloc_setup(dev, &base);
    if (rc != SPH_OK) return rc;
    double *box = reinterpret_cast<double *>(base + OFF_BOX);
    double *rb = reinterpret_cast<double *>(base + OFF_RB);
    uint64_t *ka = reinterpret_cast<uint64_t *>(base + OFF_K0), *kb = reinterpret_cast<uint64_t *>(base + OFF_K1);
    uint32_t *va = reinterpret_cast<uint32_t *>(base + OFF_V0), *vb = reinterpret_cast<uint32_t *>(base + OFF_V1);
    uint32_t *hist = reinterpret_cast<uint32_t *>(base + OFF_HIST), *hoff = reinterpret_cast<uint32_t *>(base + OFF_HOFF);
    int *part = reinterpret_cast<int *>(base + OFF_PART);
    int *err = reinterpret_cast<int *>(base + OFF_ERR);
    const int nn = (int)n;
    // the error word is the one part of the array that must start at zero
    if (cudaMemsetAsync(err, 0, sizeof(int), st) != cudaSuccess) {
        cudaGetLastError();
        return SPH_ERR_CUDA;
    }
    // root cube and keys exactly as the octree build does (theta does not enter the keys)
    k_bbox_partial<<<NA_BOX, 256, 0, st>>>(x, y, z, nn, box);
    k_bbox_final<<<1, 256, 0, st>>>(box, NA_BOX, 0.5, rb);
    k_keys<<<(nn + 255) / 256, 256, 0, st>>>(x, y, z, nn, rb, ka, va, err);
    // stable LSD radix sort, 8 passes of 8 bits
    const int nb = (nn + NA_TILE - 1) / NA_TILE;
    const LenArg L{nullptr, 256 * nb, 0};
    for (int pass = 0; pass < 8; ++pass) {
        const int shift = pass * 8;
        k_rs_hist<<<nb, 256, 0, st>>>(ka, nn, shift, hist, nb, nullptr);
        k_scan_reduce<<<NA_SCAN, 256, 0, st>>>(reinterpret_cast<const int *>(hist), L, part);
        k_scan_part<<<1, NA_SCAN, 0, st>>>(part, NA_SCAN, nullptr);
        k_scan_down<<<NA_SCAN, 256, 0, st>>>(reinterpret_cast<const int *>(hist), reinterpret_cast<int *>(hoff), L,
                                             part);
        k_rs_scatter<<<nb, 256, 0, st>>>(ka, va, kb, vb, nn, shift, hoff, nb, nullptr);
        uint64_t *tk = ka;
        ka = kb;
        kb = tk;
        uint32_t *tv = va;
        va = vb;
        vb = tv;
    }
    if (cudaGetLastError() != cudaSuccess) return SPH_ERR_CUDA;
    if (cudaMemcpyAsync(keys_out, ka, sizeof(uint64_t) * nn, cudaMemcpyDeviceToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(order_out, va, sizeof(uint32_t) * nn, cudaMemcpyDeviceToDevice, st) != cudaSuccess) {
        cudaGetLastError();
        return SPH_ERR_CUDA;
    }
    if (capturing) return SPH_OK;   // recorded; a replay's status is not read back
    int herr = 0;
    if (cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        cudaGetLastError();
        return SPH_ERR_CUDA;
    }
    return (herr & ERR_NONFINITE) ? SPH_ERR_NONFINITE : SPH_OK;
}
