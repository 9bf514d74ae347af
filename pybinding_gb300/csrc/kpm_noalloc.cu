// Diagonal KPM moments without any device allocation.
//
// Some callers cannot let a library allocate device memory: cudaMalloc and
// cudaFree may synchronize the whole device (stalling other streams in a
// latency-critical loop), and frameworks that own all device memory through
// their own pool, or run under a fixed memory budget, cannot accept hidden
// allocations. This entry point serves them: the caller passes every input
// and output buffer, and the scratch the recursion needs (the per-step moment
// sums and the tile list) lives in one file-scope device array of fixed size.
//
// The array is a static __device__ object, so every GPU that loads this
// library holds it until the process exits, and every call shares it: calls
// that overlap on the GPU (from different streams or threads) race on it.
#include "kpm_gb300.h"
#include "kpm_internal.h"

#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>
#include <string>

namespace {

// 4 MiB of scratch: the tile list (16 bytes per tile) followed by the FP64 moment
// sums of every step ((M / 2) * K * sums-per-vector doubles).
constexpr size_t kScratchBytes = size_t{4} << 20;
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_ptr[kMaxDevices] = {};

__global__ void fill_tiles_kernel(kpm::Tile* tiles, int num_tiles, int32_t rows, int32_t rows_per_tile) {
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= num_tiles) return;
    int32_t const b = i * rows_per_tile;
    tiles[i] = kpm::Tile{b, min(rows, b + rows_per_tile), 0, 0};
}

int fail(int code, std::string const& msg) {
    kpm::set_last_error(msg);  // reported by kpm_last_error(), like every other entry point
    return code;
}

// Host code cannot use the array's name as a device address: look it up once per
// device, with that device current.
int scratch_address(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(KPM_ERR_CUDA, std::string("cudaGetDevice failed: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(KPM_ERR_CUDA, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (g_scratch_ptr[dev] == nullptr) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess || p == nullptr)
            return fail(KPM_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch) failed: ") + cudaGetErrorString(e));
        g_scratch_ptr[dev] = p;
    }
    *out = g_scratch_ptr[dev];
    return KPM_OK;
}

}  // namespace

extern "C" int kpm_moments_diag_noalloc(int32_t vector_type, int64_t rows, int32_t width, const int32_t* col,
                                        const void* val, int64_t num_vectors, void* r0, void* r1,
                                        int64_t num_moments, double* out, void* stream) {
    if (vector_type < KPM_F32 || vector_type > KPM_C128) return fail(KPM_ERR_VALUE, "unknown vector type");
    if (rows < 1 || rows > (int64_t{1} << 30)) return fail(KPM_ERR_VALUE, "rows must be in [1, 2^30]");
    if (width < 1) return fail(KPM_ERR_VALUE, "width must be >= 1");
    if (!col || !val || !r0 || !r1 || !out) return fail(KPM_ERR_VALUE, "null device pointer");
    if (num_moments < 2 || num_moments % 2 != 0) return fail(KPM_ERR_VALUE, "num_moments must be even and >= 2");
    int const vb = kpm::vtype_bytes(vector_type);
    int const e16 = 16 / vb;
    int E = 1, LPR = 1;
    if (num_vectors != 1) {
        E = e16;
        LPR = static_cast<int>(num_vectors / e16);
        if (num_vectors % e16 != 0 || !kpm::diag_shape_supported(vector_type, E, LPR))
            return fail(KPM_ERR_VALUE, "num_vectors must be 1 or a block width with 32..512 bytes per row "
                                       "(a multiple of 16 bytes, power-of-two lanes)");
    }
    int const K = E * LPR;
    int const NV = kpm::vtype_nv(vector_type);
    int const rows_per_tile = (256 / LPR) * 8;
    int64_t const num_tiles = (rows + rows_per_tile - 1) / rows_per_tile;
    int64_t const half = num_moments / 2;
    size_t const tile_bytes = ((static_cast<size_t>(num_tiles) * sizeof(kpm::Tile) + 255) / 256) * 256;
    size_t const step_doubles = static_cast<size_t>(K) * NV;
    size_t const sum_bytes = sizeof(double) * step_doubles * static_cast<size_t>(half);
    if (tile_bytes + sum_bytes > kScratchBytes) {
        char msg[256];
        std::snprintf(msg, sizeof msg,
                      "problem too large for the fixed scratch: needs %zu bytes (tiles %zu + moment sums %zu), "
                      "limit %zu bytes; use kpm_moments_diag, or fewer moments or vectors per call",
                      tile_bytes + sum_bytes, tile_bytes, sum_bytes, kScratchBytes);
        return fail(KPM_ERR_VALUE, msg);
    }
    auto s = static_cast<cudaStream_t>(stream);
    if (s != nullptr) {  // the scratch address below is the current device's: the stream must be on it
        int sdev = -1, cur = -1;
        cudaError_t const e1 = cudaStreamGetDevice(s, &sdev);
        cudaError_t const e2 = cudaGetDevice(&cur);
        if (e1 != cudaSuccess || e2 != cudaSuccess)
            return fail(KPM_ERR_CUDA, std::string("cannot read the stream's device: ") +
                                          cudaGetErrorString(e1 != cudaSuccess ? e1 : e2));
        if (sdev != cur) return fail(KPM_ERR_VALUE, "the stream belongs to another device than the current one");
    }
    void* base = nullptr;
    int rc = scratch_address(&base);
    if (rc != KPM_OK) return rc;
    auto* tiles = static_cast<kpm::Tile*>(base);
    auto* sums = reinterpret_cast<double*>(static_cast<unsigned char*>(base) + tile_bytes);

#define NOALLOC_CUDA(expr)                                                                                  \
    do {                                                                                                    \
        cudaError_t e_ = (expr);                                                                            \
        if (e_ != cudaSuccess) return fail(KPM_ERR_CUDA, std::string("CUDA error: ") + cudaGetErrorString(e_) + " at " #expr); \
    } while (0)

    fill_tiles_kernel<<<static_cast<unsigned>((num_tiles + 127) / 128), 128, 0, s>>>(
        tiles, static_cast<int>(num_tiles), static_cast<int32_t>(rows), rows_per_tile);
    NOALLOC_CUDA(cudaGetLastError());
    // the array keeps the previous call's sums: clear them
    NOALLOC_CUDA(cudaMemsetAsync(sums, 0, sum_bytes, s));

    kpm::DiagStep a{};
    a.vtype = vector_type;
    a.E = E;
    a.LPR = LPR;
    a.col = col;
    a.val = val;
    a.W = width;
    a.batch_stride = rows * K;
    a.tiles = tiles;
    a.num_tiles = static_cast<int>(num_tiles);
    a.row_limit = static_cast<int32_t>(rows);
    a.nbatch = 1;
    a.unroll = 1;
    a.x = r0;
    a.y = r1;
    a.acc = sums;
    a.init = true;
    NOALLOC_CUDA(kpm::launch_diag_step(a, s));
    a.init = false;
    void* x = r1;
    void* y = r0;
    for (int64_t n = 2; n <= half; ++n) {
        a.x = x;
        a.y = y;
        a.acc = sums + step_doubles * (n - 1);
        NOALLOC_CUDA(kpm::launch_diag_step(a, s));
        void* t = x;
        x = y;
        y = t;
    }
    NOALLOC_CUDA(kpm::launch_collect_diag(vector_type, sums, 1, 1, K, half, num_moments, num_vectors, false, out, s));
#undef NOALLOC_CUDA
    return KPM_OK;
}
