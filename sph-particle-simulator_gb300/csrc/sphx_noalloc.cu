// sphx_density_noalloc: the density + pressure evaluation for callers that must not
// allocate device memory.
//
// Some host applications own every byte of device memory: an engine or visualiser that
// embeds the SPH step reserves a fixed budget up front and hands libraries pointers into
// it, and in a per-frame loop a cudaMalloc/cudaFree would also synchronise the device and
// stall the frame.  Those callers cannot use the context API (sphx_create allocates the
// step's buffers).  This entry point takes device pointers for its inputs and outputs and
// keeps all of its working memory -- packed and cell-sorted particle copies, radix-sort
// keys and permutation, the cell grid, the tile list, the device-side step state -- in
// one file-scope __device__ array of fixed size (kNoAllocScratchBytes, about 8 MiB),
// which every GPU that loads the library holds until the process exits.  It runs the same
// kernels as sphx_eval's grid build and density pass, so its results are those of
// sphx_eval + sphx_download.
//
// Limits and rules (also in include/sphx.h):
//  - at most SPHX_NOALLOC_MAX_PARTICLES particles per call; larger n is rejected with
//    SPHX_ERR_CAPACITY before anything is launched;
//  - the cell grid has SPHX_NOALLOC_MAX_CELLS cells; a larger box of occupied cells is
//    folded onto it (results unchanged, more candidates to test);
//  - all calls share the one array, which keeps the previous call's contents: the
//    device-side step state is cleared at the start of every call, every other region is
//    fully written before it is read.  Calls whose work overlaps on the GPU (two streams,
//    two host threads) race on the array and must be serialised by the caller;
//  - the first call on a device looks up the array's device address
//    (cudaGetSymbolAddress) with that device current; make that first call before any
//    stream capture begins.  The address is kept for the life of the process: calls
//    after a cudaDeviceReset (or any other teardown of the device's primary context) are
//    not supported;
//  - the call does not synchronise, so an error a kernel records on the device is not
//    returned; when one occurs rho and pressure are left as they were;
//  - the smoothing kernel is always the cubic spline (the reference engine's).
#include <cmath>
#include <mutex>

#include "sphx_internal.cuh"

using namespace sphx;

namespace {

constexpr size_t kAlign = 256;
constexpr size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

constexpr size_t kN = SPHX_NOALLOC_MAX_PARTICLES;
constexpr size_t kCells = SPHX_NOALLOC_MAX_CELLS;
constexpr size_t kRadixBlocks = (kN + kRadixTileN - 1) / kRadixTileN;
constexpr size_t kHist = kRadixBlocks * kRadixBuckets;
constexpr size_t kScanPart =
    ((kHist + kScanTileN - 1) / kScanTileN > (kN + kScanTileN - 1) / kScanTileN
         ? (kHist + kScanTileN - 1) / kScanTileN
         : (kN + kScanTileN - 1) / kScanTileN) + 1;

// byte offsets of the regions inside the scratch array
constexpr size_t kOffState = 0;
constexpr size_t kOffPos4 = kOffState + align_up(sizeof(DevState));
constexpr size_t kOffVel4 = kOffPos4 + align_up(kN * sizeof(float4));
constexpr size_t kOffPos4s = kOffVel4 + align_up(kN * sizeof(float4));
constexpr size_t kOffVel4s = kOffPos4s + align_up(kN * sizeof(float4));
constexpr size_t kOffAux4s = kOffVel4s + align_up(kN * sizeof(float4));
constexpr size_t kOffKey0 = kOffAux4s + align_up(kN * sizeof(float4));
constexpr size_t kOffKey1 = kOffKey0 + align_up(kN * sizeof(uint32_t));
constexpr size_t kOffVal0 = kOffKey1 + align_up(kN * sizeof(uint32_t));
constexpr size_t kOffVal1 = kOffVal0 + align_up(kN * sizeof(uint32_t));
constexpr size_t kOffKeyS = kOffVal1 + align_up(kN * sizeof(uint32_t));
constexpr size_t kOffIdS = kOffKeyS + align_up(kN * sizeof(uint32_t));
constexpr size_t kOffTiles = kOffIdS + align_up(kN * sizeof(uint32_t));
constexpr size_t kOffOff = kOffTiles + align_up(kN * sizeof(uint32_t));
constexpr size_t kOffHist = kOffOff + align_up((kCells + 2) * sizeof(uint32_t));
constexpr size_t kOffScan = kOffHist + align_up(kHist * sizeof(uint32_t));
constexpr size_t kNoAllocScratchBytes = kOffScan + align_up(kScanPart * sizeof(uint32_t));

// The scratch.  In host code this name is only a host-side stand-in for the device
// array: its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned char* g_scratch_addr[kMaxDevices] = {};
int g_num_sms[kMaxDevices] = {};

// Looks up (once per device, with that device current) the device address of the
// scratch array and the SM count.
int setup_device(int dev, unsigned char** addr, int* sms) {
    if (dev < 0 || dev >= kMaxDevices) return SPHX_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p)
            return SPHX_ERR_CUDA;
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            return SPHX_ERR_CUDA;
        g_num_sms[dev] = n > 0 ? n : 1;
        g_scratch_addr[dev] = static_cast<unsigned char*>(p);
    }
    *addr = g_scratch_addr[dev];
    *sms = g_num_sms[dev];
    return SPHX_OK;
}

// rho and P of the sorted particles back to the caller's arrays in insertion order --
// skipped entirely when a kernel of this call recorded a device-side error, so that the
// caller's buffers keep what they held instead of a partial result.
__global__ void k_noalloc_unpack(int n, const DevState* __restrict__ ds,
                                 const uint32_t* __restrict__ id_s,
                                 const float4* __restrict__ aux4_s, float* __restrict__ rho,
                                 float* __restrict__ pressure) {
    if (ds->status) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t id = id_s[i];
        const float4 a = aux4_s[i];
        if (rho) rho[id] = a.x;
        if (pressure) pressure[id] = a.y;
    }
}

}  // namespace

extern "C" int sphx_density_noalloc(const sphx_params* p, size_t n, const float* pos_xyz,
                                    const float* mass, float* rho, float* pressure,
                                    void* cuda_stream) {
    if (!p) return SPHX_ERR_INVALID_ARG;
    if (n > kN) return SPHX_ERR_CAPACITY;
    if (n == 0) return SPHX_OK;
    if (!pos_xyz || !mass || (!rho && !pressure)) return SPHX_ERR_INVALID_ARG;
    const float r = p->neighbor_search_radius;
    if (!(r > 0.0f) || !std::isfinite(r) || !std::isfinite(1.0f / r)) return SPHX_ERR_INVALID_ARG;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return SPHX_ERR_CUDA;
    unsigned char* base = nullptr;
    int sms = 0;
    int rc = setup_device(dev, &base, &sms);
    if (rc) return rc;

    // the step constants of sphx_set_params + sphx_eval on a context with the default
    // (cubic-spline) kernel in exact mode: this entry point always uses the cubic spline
    StepConst c{};
    step_const_from_params(*p, n, SPHX_KERNEL_CUBIC_SPLINE, SPHX_MODE_EXACT, (uint32_t)kCells, c);

    Buffers b{};
    b.pos4 = reinterpret_cast<float4*>(base + kOffPos4);
    b.vel4 = reinterpret_cast<float4*>(base + kOffVel4);
    b.pos4_s = reinterpret_cast<float4*>(base + kOffPos4s);
    b.vel4_s = reinterpret_cast<float4*>(base + kOffVel4s);
    b.aux4_s = reinterpret_cast<float4*>(base + kOffAux4s);
    b.acc4_s = nullptr;  // not touched by the grid build or the density pass
    b.key[0] = reinterpret_cast<uint32_t*>(base + kOffKey0);
    b.key[1] = reinterpret_cast<uint32_t*>(base + kOffKey1);
    b.val[0] = reinterpret_cast<uint32_t*>(base + kOffVal0);
    b.val[1] = reinterpret_cast<uint32_t*>(base + kOffVal1);
    b.key_s = reinterpret_cast<uint32_t*>(base + kOffKeyS);
    b.id_s = reinterpret_cast<uint32_t*>(base + kOffIdS);
    b.tile_start = reinterpret_cast<uint32_t*>(base + kOffTiles);
    b.off = reinterpret_cast<uint32_t*>(base + kOffOff);
    b.hist = reinterpret_cast<uint32_t*>(base + kOffHist);
    b.scan_part = reinterpret_cast<uint32_t*>(base + kOffScan);
    b.diag_part = nullptr;
    b.radix_blocks = (int)kRadixBlocks;
    b.scan_part_cap = (int)kScanPart;
    b.diag_blocks = 0;
    DevState* ds = reinterpret_cast<DevState*>(base + kOffState);

    LaunchCtx L{};
    L.stream = static_cast<cudaStream_t>(cuda_stream);
    L.device = dev;
    L.num_sms = sms;
    L.warps_per_block = 4;
    L.blocks_per_sm = 0;

    // the previous call's device-side state must not leak into this one
    if (cudaMemsetAsync(ds, 0, sizeof(DevState), L.stream) != cudaSuccess) return SPHX_ERR_CUDA;
    launch_pack(L, (int)n, pos_xyz, nullptr, mass, b.pos4, b.vel4);
    launch_begin_step(L, ds, 1);
    launch_build_grid(L, c, b, ds);
    launch_density(L, c, b, ds);
    const int ub = (int)((n + 255) / 256) < 4 * sms ? (int)((n + 255) / 256) : 4 * sms;
    k_noalloc_unpack<<<ub, 256, 0, L.stream>>>((int)n, ds, b.id_s, b.aux4_s, rho, pressure);
    if (cudaGetLastError() != cudaSuccess) return SPHX_ERR_CUDA;
    return SPHX_OK;
}
