// gs_knn_binned_noalloc: the binned self-KNN for callers that cannot allocate
// device memory.
//
// Some callers own every byte of device memory themselves and cannot let a
// library call cudaMalloc: code running inside a pre-sized memory pool (a
// game engine or simulator frame allocator, a framework's caching
// allocator), code that must not allocate once a real-time loop has started,
// or code that wraps the call in its own allocation accounting.  For them
// this entry point takes the positions and the output arrays from the caller
// and keeps its working memory (per-cell counts and starts, scan partials,
// per-agent cell and rank, the bucketed positions) in one fixed array that
// is part of the library image.
//
// The array (kScratchBytes, 32 MiB) is reserved on every GPU that loads the
// library and stays reserved until the process exits.  A call needs
//   8 * (cells + 1) + 4 * ceil(cells / 4096) + 28 * n bytes + up to 1.5 KiB of
// alignment, so it holds for example 800,000 agents on a 1,048,576-cell grid
// (a 128 x 64 x 128 world); larger problems are rejected with
// GS_ERR_INVALID_ARG.
//
// Every call uses the same array and leaves its contents behind; the cell
// counts, which must start at zero, are cleared by each call.  Calls whose
// work overlaps on the GPU (several streams, or several host threads) race on
// the array and must be serialised by the caller.
//
// The array's device address is looked up with cudaGetSymbolAddress the first
// time a call is made in a CUDA context (with that context's device current)
// and kept for that context only: a context created later on the same device
// (after cudaDeviceReset, say) loads the library's module again, possibly at
// another address, and its first call looks the address up again.  Make the
// first call on each device, and the first after a reset, before starting any
// stream capture on that device.
#include <cuda.h>

#include <cmath>
#include <cstdint>
#include <mutex>

#include "gs_launch.h"

namespace gs {
namespace {

constexpr size_t kScratchBytes = size_t(32) << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_knn_scratch[kScratchBytes];

std::mutex g_mu;
// Per device: the context the address was looked up in (0: none) and the address.
unsigned long long g_scratch_ctx[kMaxDevices] = {};
void* g_scratch_addr[kMaxDevices] = {};

// cuCtxGetCurrent / cuCtxGetId through the runtime's driver entry points (the
// library links the static runtime, not libcuda).  Null when unavailable.
using CtxGetCurrent = CUresult (*)(CUcontext*);
using CtxGetId = CUresult (*)(CUcontext, unsigned long long*);
CtxGetCurrent g_ctx_current = nullptr;
CtxGetId g_ctx_id = nullptr;
std::once_flag g_entry_once;

void resolve_entry_points() {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
        g_ctx_current = reinterpret_cast<CtxGetCurrent>(f);
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
        g_ctx_id = reinterpret_cast<CtxGetId>(f);
}

// Unique id of the calling thread's current context, 0 if none is current or
// the driver cannot say.
unsigned long long current_context_id() {
    if (!g_ctx_current || !g_ctx_id) return 0;
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (g_ctx_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
    if (g_ctx_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Device address of g_knn_scratch in the current context of the current
// device: looked up once per context, again whenever the context changed.
gs_status scratch_address(void** out) {
    std::call_once(g_entry_once, resolve_entry_points);
    int dev = 0;
    GS_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return fail(GS_ERR_UNSUPPORTED, "device index too large");
    std::lock_guard<std::mutex> lock(g_mu);
    const unsigned long long ctx = current_context_id();
    if (ctx == 0 || ctx != g_scratch_ctx[dev] || !g_scratch_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_knn_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(knn scratch)");
        // the lookup made the device's primary context current if none was
        g_scratch_ctx[dev] = current_context_id();
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return GS_OK;
}

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace
}  // namespace gs

using namespace gs;

extern "C" gs_status gs_knn_binned_noalloc(const float* positions4, unsigned n,
                                           const unsigned world_cells[3],
                                           const float world_size[3], unsigned search_radius,
                                           unsigned k, unsigned* idx_out, float* dist_out,
                                           void* stream) {
    if (!world_cells || !world_size) return fail(GS_ERR_INVALID_ARG, "null grid");
    if (n > 0 && (!positions4 || !idx_out || !dist_out))
        return fail(GS_ERR_INVALID_ARG, "null device array");
    if (k == 0 || k > kMaxK) return fail(GS_ERR_INVALID_ARG, "k must be in 1..64");
    Grid grid;
    unsigned long long cells = 1;
    for (int a = 0; a < 3; ++a) {
        if (world_cells[a] == 0 || !(world_size[a] > 0.f) || !std::isfinite(world_size[a]))
            return fail(GS_ERR_INVALID_ARG, "bad world size or cell count");
        grid.wc[a] = world_cells[a];
        grid.ws[a] = world_size[a];
        // checked after every factor: the running product stays below 2^62
        cells *= world_cells[a];
        if (cells > (1ull << 30)) return fail(GS_ERR_INVALID_ARG, "too many cells");
    }
    const unsigned C = unsigned(cells);
    const unsigned T = scan_tile_count(C);
    // layout inside the fixed array
    const size_t o_count = 0;
    const size_t o_start = align256(o_count + size_t(C) * 4);
    const size_t o_tile = align256(o_start + (size_t(C) + 1) * 4);
    const size_t o_cell = align256(o_tile + (size_t(T) + 1) * 4);
    const size_t o_rank = align256(o_cell + size_t(n) * 4);
    const size_t o_sorted = align256(o_rank + size_t(n) * 4);
    const size_t o_pos = align256(o_sorted + size_t(n) * 4);
    const size_t need = o_pos + size_t(n) * 16;
    if (need > kScratchBytes)
        return fail(GS_ERR_INVALID_ARG,
                    "problem too large for the fixed 32 MiB KNN work array (needs " +
                        std::to_string(need) + " bytes); use gs_find_knn");
    void* base = nullptr;
    GS_TRY(scratch_address(&base));
    unsigned char* b = static_cast<unsigned char*>(base);
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    Database db;
    db.cells = C;
    db.count = reinterpret_cast<unsigned*>(b + o_count);
    db.start = reinterpret_cast<unsigned*>(b + o_start);
    db.tile = reinterpret_cast<unsigned*>(b + o_tile);
    db.cell = reinterpret_cast<unsigned*>(b + o_cell);
    db.rank = reinterpret_cast<unsigned*>(b + o_rank);
    db.sorted = reinterpret_cast<unsigned*>(b + o_sorted);
    db.pos_id = reinterpret_cast<float4*>(b + o_pos);
    // the counts must start at zero whatever an earlier call left behind
    GS_CUDA(cudaMemsetAsync(db.count, 0, size_t(C) * 4, st));
    GS_TRY(db_build(db, reinterpret_cast<const float4*>(positions4), n, grid, st));
    GS_TRY(launch_knn_binned(db, n, db, true, search_radius, k, idx_out, dist_out, st));
    return GS_OK;
}
