// noalloc.cu — Morton sort that allocates no device memory.
//
// apic_morton_sort_noalloc computes the same Morton keys and stable sort
// permutation as the handle-based sort (the APIC_STAGE_SORT stage), but for
// callers that cannot allocate device memory: code that records work into a
// stream capture, where cudaMalloc is not allowed, and host applications
// whose device memory is owned by another runtime or a fixed budget, so that
// no library call may grow it.  The caller passes device buffers for the
// positions and for the sorted keys and slots; every intermediate buffer of
// the radix sort lives in one file-scope device array of fixed size, which
// every GPU that loads this library holds until the process exits.
#include <cuda_runtime.h>

#include <mutex>
#include <vector>

#include "apic_device.cuh"
#include "apic_internal.h"

namespace apic {
namespace {

// Largest particle count the scratch array supports.
constexpr uint32_t kNoAllocMaxKeys = 1u << 20;  // 1,048,576 particles
constexpr uint32_t kNoAllocBlocks = kNoAllocMaxKeys / kSortTile;
constexpr uint32_t kHistWords = 256u * kNoAllocBlocks;
constexpr uint32_t kScanWords = (kHistWords + 1023u) / 1024u + 1u;
// layout: alternate keys | alternate slots | digit histogram | scan partials
constexpr size_t kScratchWords = 2ull * kNoAllocMaxKeys + kHistWords + kScanWords;  // ~8.5 MiB

static __device__ __align__(256) uint32_t g_sort_scratch[kScratchWords];

// Device address of the scratch array in the current CUDA context.  In host
// code the array's name only stands in for the symbol; kernels must receive
// this address.  It is looked up with cudaGetSymbolAddress once per context
// (normally once per device: the runtime's primary context) and cached under
// the context's unique id, so a context created later (after
// cudaDeviceReset, or a caller's own context) gets its own lookup instead of
// a stale address.
struct ScratchEntry {
    unsigned long long ctx;
    uint32_t* addr;
};
std::mutex g_setup_mutex;
std::vector<ScratchEntry> g_scratch;

cudaError_t scratch_for_current_context(uint32_t** out) {
    unsigned long long ctx = 0;
    cudaError_t e = current_context_key(&ctx);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    for (const ScratchEntry& s : g_scratch)
        if (s.ctx == ctx) {
            *out = s.addr;
            return cudaSuccess;
        }
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_sort_scratch);
    if (e != cudaSuccess) return e;
    g_scratch.push_back({ctx, static_cast<uint32_t*>(p)});
    *out = static_cast<uint32_t*>(p);
    return cudaSuccess;
}

// Morton key of each particle's clamped cell and its slot (src/apic.rs:1049-1064).
__global__ void k_keys_from_positions(const float* __restrict__ px, const float* __restrict__ py, uint32_t n,
                                      float dx, float max_x, float max_y, uint32_t* __restrict__ keys,
                                      uint32_t* __restrict__ vals) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float gx = px[i] / dx, gy = py[i] / dx;
    uint32_t cx = uint32_t(trunc_x86(fmin_x86(fmax_x86(gx, 0.0f), max_x)));
    uint32_t cy = uint32_t(trunc_x86(fmin_x86(fmax_x86(gy, 0.0f), max_y)));
    keys[i] = morton(cx, cy);
    vals[i] = i;
}

int reject(int code, const char* msg) {
    set_last_error(msg);
    return code;
}

}  // namespace
}  // namespace apic

using namespace apic;

extern "C" int apic_morton_sort_noalloc(const float* pos_x, const float* pos_y, uint32_t n, uint32_t width,
                                        uint32_t height, float cell_size, uint32_t* keys_out, uint32_t* vals_out,
                                        void* stream) {
    if (n > kNoAllocMaxKeys)
        return reject(APIC_ERR_INVALID_ARG, "apic_morton_sort_noalloc: more than 1048576 particles (scratch limit)");
    if (width == 0 || height == 0 || !(cell_size > 0.0f))
        return reject(APIC_ERR_INVALID_ARG, "apic_morton_sort_noalloc: width, height and cell_size must be positive");
    if (width > 65536u || height > 65536u)
        return reject(APIC_ERR_INVALID_ARG, "apic_morton_sort_noalloc: width and height are limited to 65536");
    if (n == 0) return APIC_OK;
    if (!pos_x || !pos_y || !keys_out || !vals_out)
        return reject(APIC_ERR_INVALID_ARG, "apic_morton_sort_noalloc: null buffer");
    uint32_t* scratch = nullptr;
    cudaError_t e = scratch_for_current_context(&scratch);
    if (e != cudaSuccess) return reject(APIC_ERR_CUDA, cudaGetErrorString(e));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    uint32_t* keys_alt = scratch;
    uint32_t* vals_alt = scratch + kNoAllocMaxKeys;
    uint32_t* hist = scratch + 2ull * kNoAllocMaxKeys;
    uint32_t* scan_tmp = hist + kHistWords;
    float max_x = float(width - 1), max_y = float(height - 1);
    k_keys_from_positions<<<div_up(n, 256), 256, 0, st>>>(pos_x, pos_y, n, cell_size, max_x, max_y, keys_out,
                                                          vals_out);
    e = radix_sort_pairs_in(keys_out, vals_out, keys_alt, vals_alt, hist, scan_tmp, n,
                            morton_key_bits(width, height), st);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return reject(APIC_ERR_CUDA, cudaGetErrorString(e));
    return APIC_OK;
}
