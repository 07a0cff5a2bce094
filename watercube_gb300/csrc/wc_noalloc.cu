// wc_noalloc.cu — the cell sort as one call that allocates nothing.
//
// Some callers cannot allocate device memory when they need a sort: a render or physics frame
// loop where cudaMalloc would synchronise the GPU and stall the frame, or a host application
// whose device memory budget is fixed up front by its own allocator. wc_sort_cells_noalloc
// serves them: the caller passes the particle positions and the output arrays, and every
// scratch buffer the sort needs lives in one file-scope device array of fixed size, reserved
// when the library is loaded and held by every GPU that loads it until the process exits.
//
// It runs the same four kernels as wc_fluid_sort (bin_count, scan_cells, scatter_cells,
// rank_gather) and gives the same keys, permutation, cell table and sorted positions.
//
// Rules of use:
//   * Limits: at most WC_NOALLOC_MAX_PARTICLES particles and WC_NOALLOC_MAX_CELLS cells
//     (grid_res^3); larger requests are rejected with WC_ERR_INVALID_ARG.
//   * The first call on a device looks up the array's device address (cudaGetSymbolAddress)
//     with that device current; make that first call before any stream capture.
//   * All calls share the one array. Calls whose work overlaps on the GPU (different streams
//     without ordering between them, or different host threads) race on it; order them.
//   * Each call clears the part of the array that must start at zero (the histogram and the
//     error word); the rest keeps the last call's contents.
//   * Device-side errors (a non-finite position, a scan wait that ran out, a cell beyond
//     MAX_SORT_CELL_PARTICLES) are recorded in the array's error word and not seen by the call,
//     which only enqueues work. wc_sort_cells_noalloc_status(stream) waits for the stream and
//     reports them for the last call; the word is cleared by the next call.
#include <cuda_runtime.h>

#include <mutex>

#include "wc_internal.h"
#include "wc_util.h"

namespace {

constexpr uint32_t MAXP = WC_NOALLOC_MAX_PARTICLES;
constexpr uint32_t MAXC = WC_NOALLOC_MAX_CELLS;
constexpr uint32_t MAX_TILES = (MAXC + wc::SCAN_TILE - 1) / wc::SCAN_TILE;

constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Byte layout of the scratch array.
constexpr size_t OFF_RANKS = 0;
constexpr size_t OFF_UNORDERED = align256(OFF_RANKS + sizeof(uint32_t) * MAXP);
constexpr size_t OFF_COUNTS = align256(OFF_UNORDERED + sizeof(uint32_t) * MAXP);
constexpr size_t OFF_CELL_LIST = align256(OFF_COUNTS + sizeof(uint32_t) * MAXC);
constexpr size_t OFF_DESC = align256(OFF_CELL_LIST + sizeof(uint32_t) * MAXC);
constexpr size_t OFF_WORDS = align256(OFF_DESC + sizeof(unsigned long long) * MAX_TILES);
constexpr size_t SCRATCH_BYTES = align256(OFF_WORDS + 4 * sizeof(uint32_t));  // tile counter, non-empty count, error

static __device__ __align__(256) unsigned char g_sort_scratch[SCRATCH_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_setup_mutex;
unsigned char* g_scratch_addr[MAX_DEVICES] = {};
wc::LaunchDims g_dims[MAX_DEVICES];

// Once per device, with that device current: the array's device address (host code may not use
// the symbol itself — in host code it names a host-side stand-in, not device memory).
wc_status scratch_for_device(int dev, unsigned char** out, wc::LaunchDims* dims) {
    if (dev < 0 || dev >= MAX_DEVICES) return wc::fail(WC_ERR_UNSUPPORTED, "device %d beyond %d", dev, MAX_DEVICES);
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_sort_scratch);
        if (e != cudaSuccess || !p)
            return wc::fail(WC_ERR_CUDA, "cudaGetSymbolAddress of the sort scratch failed: %s", cudaGetErrorString(e));
        g_dims[dev] = wc::compute_launch_dims(dev);
        g_scratch_addr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_scratch_addr[dev];
    *dims = g_dims[dev];
    return WC_OK;
}

}  // namespace

extern "C" {

WC_API wc_status wc_sort_cells_noalloc(const void* d_positions, uint32_t n, uint32_t grid_res, float bin_size,
                                       uint32_t* d_keys, uint32_t* d_permutation, uint32_t* d_cell_start,
                                       void* d_sorted_positions, void* stream) {
    wc::clear_error();
    if (n > MAXP)
        return wc::fail(WC_ERR_INVALID_ARG, "wc_sort_cells_noalloc: %u particles exceed the limit of %u", n, MAXP);
    if (grid_res == 0 || grid_res > 1024 || (uint64_t)grid_res * grid_res * grid_res > MAXC)
        return wc::fail(WC_ERR_INVALID_ARG, "wc_sort_cells_noalloc: grid_res %u gives more than %u cells", grid_res,
                        MAXC);
    if (!(bin_size > 0.0f)) return wc::fail(WC_ERR_INVALID_ARG, "wc_sort_cells_noalloc: bin_size must be > 0");
    if (!d_cell_start || (n && (!d_positions || !d_keys || !d_permutation || !d_sorted_positions)))
        return wc::fail(WC_ERR_INVALID_ARG, "wc_sort_cells_noalloc: null buffer");
    int dev = 0;
    WC_CUDA_TRY(cudaGetDevice(&dev));
    unsigned char* base = nullptr;
    wc::LaunchDims ld;
    const wc_status st = scratch_for_device(dev, &base, &ld);
    if (st != WC_OK) return st;

    const uint32_t C = grid_res * grid_res * grid_res;
    wc::DevBuffers d{};
    d.n = n;
    d.num_cells = C;
    d.num_tiles = (C + wc::SCAN_TILE - 1) / wc::SCAN_TILE;
    d.pos_a = const_cast<float4*>(static_cast<const float4*>(d_positions));
    d.vel_a = nullptr;  // positions only: the gather skips the velocity stream
    d.pos_b = static_cast<float4*>(d_sorted_positions);
    d.vel_b = nullptr;
    d.keys = d_keys;
    d.perm = d_permutation;
    d.start = d_cell_start;
    d.ranks = reinterpret_cast<uint32_t*>(base + OFF_RANKS);
    d.unordered = reinterpret_cast<uint32_t*>(base + OFF_UNORDERED);
    d.counts = reinterpret_cast<uint32_t*>(base + OFF_COUNTS);
    d.cell_list = reinterpret_cast<uint32_t*>(base + OFF_CELL_LIST);
    d.scan_desc = reinterpret_cast<unsigned long long*>(base + OFF_DESC);
    uint32_t* words = reinterpret_cast<uint32_t*>(base + OFF_WORDS);
    d.scan_tile_counter = words;
    d.num_nonempty = words + 1;
    d.err = words + 2;

    wc::SceneConsts sc{};
    sc.bin = bin_size;
    sc.R = (int32_t)grid_res;
    sc.R_magic = wc::r_magic(grid_res);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // The histogram and the error word must start at zero; earlier calls leave them dirty.
    WC_CUDA_TRY(cudaMemsetAsync(d.counts, 0, sizeof(uint32_t) * C, s));
    WC_CUDA_TRY(cudaMemsetAsync(d.err, 0, sizeof(uint32_t), s));
    wc::launch_bin_count(d, sc, ld, s);
    wc::launch_scan_cells(d, s);
    wc::launch_scatter(d, ld, s);
    wc::launch_rank_gather(d, ld, s);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return wc::fail(WC_ERR_CUDA, "wc_sort_cells_noalloc launch: %s", cudaGetErrorString(e));
    return WC_OK;
}

WC_API wc_status wc_sort_cells_noalloc_status(void* stream) {
    wc::clear_error();
    // The kernels report into the array's error word, which the caller cannot address. Copy it
    // into a host word of this thread (no allocation), after the work already on `stream`.
    thread_local uint32_t word = 0;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    WC_CUDA_TRY(cudaMemcpyFromSymbolAsync(&word, g_sort_scratch, sizeof word, OFF_WORDS + 2 * sizeof(uint32_t),
                                          cudaMemcpyDeviceToHost, s));
    WC_CUDA_TRY(cudaStreamSynchronize(s));
    if (word & wc::DEVERR_SCAN_TIMEOUT)
        return wc::fail(WC_ERR_TIMEOUT, "wc_sort_cells_noalloc: a scan tile gave up waiting; the cell table and "
                                        "permutation of that call are invalid");
    if (word & wc::DEVERR_NONFINITE)
        return wc::fail(WC_ERR_NUMERIC, "wc_sort_cells_noalloc: a non-finite position was binned (to cell 0)");
    if (word & wc::DEVERR_CELL_OVERFLOW)
        return wc::fail(WC_ERR_NUMERIC, "wc_sort_cells_noalloc: a cell held more than %u particles; its members "
                                        "were placed in arrival order", wc::MAX_SORT_CELL_PARTICLES);
    return WC_OK;
}

}  // extern "C"
