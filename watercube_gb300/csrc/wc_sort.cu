// wc_sort.cu — the counting sort by cell (the reference's Sort::run, src/core/Sort.cpp:254-267)
// as four sm_103a kernels:
//
//   bin_count     count.comp:25-36     key per particle + warp-aggregated cell histogram; the
//                                      histogram add returns an arrival rank in the cell
//   scan_cells    linearScan.comp:15-28 single-pass exclusive scan of the histogram with
//                                      decoupled look-back (a warp reads 32 predecessors per
//                                      round; bounded waits), fused with the
//                                      non-empty cell list and the histogram clear
//   scatter_cells reorder.comp:32-45   particle index -> offsets[key] + arrival rank
//   rank_gather   reorder.comp/sort.comp stable rank = #(members of the cell with a smaller
//                                      index); writes the permutation (sort.comp:44) and
//                                      gathers the SoA particle state into sorted order
//                                      (cells beyond MAX_SORT_CELL_PARTICLES: arrival order)
//
// The reference's in-cell order is whatever order atomicAdd hands out; this sort defines it as
// the input order (stable), so the permutation is reproducible and bit-exact against a serial
// counting sort.
#include <cuda_runtime.h>

#include "wc_internal.h"
#include "wc_util.h"

namespace wc {
namespace {

constexpr unsigned FULL = 0xffffffffu;

// Test hook of the look-back (wc_debug_scan_stall): its spin limit, and a switch that makes it
// poll a descriptor nothing publishes, so that every tile after the first runs its wait out.
__device__ uint32_t g_scan_spin_limit = SCAN_SPIN_LIMIT;
__device__ uint32_t g_scan_stall = 0;
constexpr unsigned long long DESC_AGG = 1ull << 62;      // tile aggregate published
constexpr unsigned long long DESC_PREFIX = 2ull << 62;   // inclusive prefix published
constexpr unsigned long long DESC_VALUE = (1ull << 62) - 1;
// Packed scan value: bits [0,31) particle count, bits [31,62) non-empty cell count.
constexpr int NZ_SHIFT = 31;
constexpr unsigned long long COUNT_MASK = (1ull << NZ_SHIFT) - 1;

// ivec3(p / binSize) then clamp(.., 0, R-1) (count.comp:32), with NaN -> 0.
__device__ __forceinline__ int32_t cell_axis(float q, int32_t R) {
    if (!(q >= 1.0f)) return 0;
    if (q >= (float)(R - 1)) return R - 1;
    return (int32_t)q;
}

__device__ __forceinline__ uint32_t cell_key(float4 p, float bin, int32_t R) {
    const int32_t cx = cell_axis(__fdiv_rn(p.x, bin), R);
    const int32_t cy = cell_axis(__fdiv_rn(p.y, bin), R);
    const int32_t cz = cell_axis(__fdiv_rn(p.z, bin), R);
    return (uint32_t)((cz * R + cy) * R + cx);  // count.comp:33
}

__device__ __forceinline__ unsigned long long ld_volatile_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.volatile.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_volatile_u64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.volatile.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// One thread per particle (grid-stride, block-uniform trip count so that every lane of a warp
// reaches the match/vote instructions together).
// BATCHED: particle slot i belongs to the scene whose slot range holds it; its key is that
// scene's cell offset plus the key in the scene's own grid.
template <bool BATCHED>
__global__ void __launch_bounds__(256) bin_count_kernel(const float4* __restrict__ pos, uint32_t n, float bin,
                                                        int32_t R, const BatchTables bt, uint32_t* __restrict__ keys,
                                                        uint32_t* __restrict__ ranks, uint32_t* __restrict__ counts,
                                                        unsigned long long* __restrict__ scan_desc,
                                                        uint32_t* __restrict__ scan_tile_counter, uint32_t num_tiles,
                                                        uint32_t* __restrict__ err) {
    __shared__ uint32_t s_poff[BATCHED ? MAX_SCENES + 1 : 1];
    __shared__ uint32_t s_coff[BATCHED ? MAX_SCENES + 1 : 1];
    __shared__ float s_bin[BATCHED ? MAX_SCENES : 1];
    __shared__ int32_t s_R[BATCHED ? MAX_SCENES : 1];
    if (BATCHED) {
        for (uint32_t t = threadIdx.x; t <= bt.num_scenes; t += blockDim.x) {
            s_poff[t] = bt.poff[t];
            s_coff[t] = bt.coff[t];
            if (t < bt.num_scenes) {
                s_bin[t] = bt.scenes[t].bin;
                s_R[t] = bt.scenes[t].R;
            }
        }
        __syncthreads();
    }
    const uint32_t gid = blockIdx.x * blockDim.x + threadIdx.x;
    // Reset the look-back state of the scan that follows this kernel on the stream.
    for (uint32_t t = gid; t < num_tiles; t += gridDim.x * blockDim.x) scan_desc[t] = 0ull;
    if (gid == 0) *scan_tile_counter = 0u;

    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t i = base + threadIdx.x;
        const bool valid = i < n;
        uint32_t key = 0;
        if (valid) {
            const float4 p = pos[i];
            if (!(isfinite(p.x) && isfinite(p.y) && isfinite(p.z))) atomicOr(err, DEVERR_NONFINITE);
            if (BATCHED) {
                const uint32_t sc = find_scene(s_poff, bt.num_scenes, i);
                key = s_coff[sc] + cell_key(p, s_bin[sc], s_R[sc]);
            } else {
                key = cell_key(p, bin, R);
            }
        }
        const unsigned vmask = __ballot_sync(FULL, valid);
        if (valid) {
            const unsigned peers = __match_any_sync(vmask, key);
            const int leader = __ffs(peers) - 1;
            uint32_t first = 0;
            if ((int)lane == leader) first = atomicAdd(&counts[key], (uint32_t)__popc(peers));
            first = __shfl_sync(peers, first, leader);
            ranks[i] = first + (uint32_t)__popc(peers & ((1u << lane) - 1u));
            keys[i] = key;
        }
    }
}

__global__ void __launch_bounds__(SCAN_THREADS) scan_cells_kernel(uint32_t* __restrict__ counts, uint32_t C,
                                                                  uint32_t* __restrict__ start,
                                                                  uint32_t* __restrict__ cell_list,
                                                                  uint32_t* __restrict__ num_nonempty,
                                                                  unsigned long long* desc, uint32_t* tile_counter,
                                                                  uint32_t num_tiles, uint32_t* err) {
    constexpr int NW = SCAN_THREADS / 32;
    __shared__ uint32_t s_tile;
    __shared__ unsigned long long s_warp[NW];
    __shared__ unsigned long long s_excl;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    // Tiles are numbered in arrival order, so every predecessor of a tile is already running:
    // the look-back below never waits on a block that has not been scheduled.
    if (tid == 0) s_tile = atomicAdd(tile_counter, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t base = tile * (uint32_t)SCAN_TILE + tid * (uint32_t)SCAN_ITEMS;

    uint32_t v[SCAN_ITEMS];
    if (base + SCAN_ITEMS <= C) {
        uint4* src = reinterpret_cast<uint4*>(counts + base);
#pragma unroll
        for (int q = 0; q < SCAN_ITEMS / 4; ++q) {
            const uint4 u = src[q];
            v[4 * q + 0] = u.x;
            v[4 * q + 1] = u.y;
            v[4 * q + 2] = u.z;
            v[4 * q + 3] = u.w;
            src[q] = make_uint4(0u, 0u, 0u, 0u);  // the histogram starts at zero next step
        }
    } else {
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; ++k) {
            const uint32_t c = base + k;
            v[k] = c < C ? counts[c] : 0u;
            if (c < C) counts[c] = 0u;
        }
    }
    unsigned long long tv = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) tv += ((unsigned long long)(v[k] != 0u) << NZ_SHIFT) | v[k];

    unsigned long long x = tv;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const unsigned long long y = __shfl_up_sync(FULL, x, off);
        if ((int)lane >= off) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        unsigned long long w = lane < NW ? s_warp[lane] : 0ull;
#pragma unroll
        for (int off = 1; off < NW; off <<= 1) {
            const unsigned long long y = __shfl_up_sync(FULL, w, off);
            if ((int)lane >= off) w += y;
        }
        if (lane < NW) s_warp[lane] = w;
    }
    __syncthreads();
    const unsigned long long tile_total = s_warp[NW - 1];
    const unsigned long long thread_excl = (warp ? s_warp[warp - 1] : 0ull) + x - tv;

    // Look-back by warp 0: lane k reads the descriptor of tile (tile - 1 - k - 32 r) in round r; the
    // window's values up to and including the nearest published prefix are summed. A lane whose
    // descriptor is not yet published (and lies before that prefix) makes the warp wait, bounded.
    if (warp == 0) {
        unsigned long long excl = 0;
        if (tile == 0) {
            if (lane == 0) st_volatile_u64(desc, DESC_PREFIX | tile_total);
        } else {
            if (lane == 0) st_volatile_u64(desc + tile, DESC_AGG | tile_total);
            const uint32_t limit = g_scan_spin_limit;
            const bool stall = g_scan_stall != 0u;
            int32_t j = (int32_t)tile - 1 - (int32_t)lane;
            uint32_t spins = 0;
            for (;;) {
                // beyond tile 0: an empty prefix, so every window ends there
                const unsigned long long d = j < 0 ? DESC_PREFIX : (stall ? 0ull : ld_volatile_u64(desc + j));
                const unsigned long long flag = d >> 62;
                const unsigned prefix = __ballot_sync(FULL, flag == 2ull);
                const unsigned missing = __ballot_sync(FULL, flag == 0ull);
                const int first = prefix ? __ffs(prefix) - 1 : 32;
                const unsigned upto = first >= 31 ? FULL : ((2u << first) - 1u);
                if (missing & upto) {
                    if (++spins > limit) {  // bounded: report and publish what we have
                        if (lane == 0) atomicOr(err, DEVERR_SCAN_TIMEOUT);
                        break;
                    }
                    __nanosleep(64);
                    continue;
                }
                unsigned long long v = (int)lane <= first ? (d & DESC_VALUE) : 0ull;
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(FULL, v, off);
                excl += v;
                if (first < 32) break;
                j -= 32;
            }
            if (lane == 0) st_volatile_u64(desc + tile, DESC_PREFIX | ((excl + tile_total) & DESC_VALUE));
        }
        if (lane == 0) s_excl = excl;
    }
    __syncthreads();
    const unsigned long long pre = s_excl + thread_excl;
    uint32_t run = (uint32_t)(pre & COUNT_MASK);
    uint32_t nz = (uint32_t)(pre >> NZ_SHIFT);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        const uint32_t c = base + k;
        if (c < C) {
            start[c] = run;
            if (v[k]) cell_list[nz++] = c;
            run += v[k];
        }
    }
    if (tile == num_tiles - 1 && tid == SCAN_THREADS - 1) {
        start[C] = run;
        *num_nonempty = nz;
    }
}

// Tables are consistent unless a scan tile timed out (reported through DEVERR_SCAN_TIMEOUT);
// the bounds checks below keep every access inside its buffer even then.
__global__ void __launch_bounds__(256) scatter_cells_kernel(uint32_t n, const uint32_t* __restrict__ keys,
                                                            const uint32_t* __restrict__ ranks,
                                                            const uint32_t* __restrict__ start,
                                                            uint32_t* __restrict__ unordered) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t dst = start[keys[i]] + ranks[i];
        if (dst < n) unordered[dst] = i;
    }
}

// VEL: also gather the velocity stream (the cell sort alone moves positions only).
// A cell of more than MAX_SORT_CELL_PARTICLES particles (a collapsed or non-finite state) takes
// its members in arrival order instead: the stable rank costs O(k) per member, O(k^2) per cell,
// and an all-NaN state puts every particle in cell 0. Arrival ranks are unique in the cell, so
// the permutation stays a permutation; the step reports the cell through DEVERR_CELL_OVERFLOW.
template <bool IDS, bool VEL>
__global__ void __launch_bounds__(256) rank_gather_kernel(uint32_t n, const uint32_t* __restrict__ keys,
                                                          const uint32_t* __restrict__ ranks,
                                                          const uint32_t* __restrict__ unordered,
                                                          const uint32_t* __restrict__ start,
                                                          const float4* __restrict__ pos_in,
                                                          const float4* __restrict__ vel_in,
                                                          const uint32_t* __restrict__ ids_in,
                                                          float4* __restrict__ pos_out, float4* __restrict__ vel_out,
                                                          uint32_t* __restrict__ ids_out, uint32_t* __restrict__ perm,
                                                          uint32_t* __restrict__ err, float* __restrict__ xyz,
                                                          uint32_t xyz_stride, float* __restrict__ vxyz) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t key = keys[i];
        const uint32_t s = start[key], e = min(start[key + 1], n);
        uint32_t r = 0;
        if (e - min(s, e) <= MAX_SORT_CELL_PARTICLES) {
            for (uint32_t q = s; q < e; ++q) r += unordered[q] < i ? 1u : 0u;
        } else {
            r = ranks[i];
            if (r == 0u) atomicOr(err, DEVERR_CELL_OVERFLOW);
        }
        const uint32_t dst = s + r;
        if (dst >= n) continue;
        perm[dst] = i;
        const float4 p = pos_in[i];
        pos_out[dst] = p;
        if (xyz) {
            xyz[dst] = p.x;
            xyz[xyz_stride + dst] = p.y;
            xyz[2 * (size_t)xyz_stride + dst] = p.z;
        }
        if (VEL && vxyz) {
            const float4 v = vel_in[i];
            vxyz[dst] = v.x;
            vxyz[xyz_stride + dst] = v.y;
            vxyz[2 * (size_t)xyz_stride + dst] = v.z;
        }
        if (VEL) vel_out[dst] = vel_in[i];
        if (IDS) ids_out[dst] = ids_in[i];
    }
}

__global__ void aos_to_soa_kernel(const float4* __restrict__ aos, float4* __restrict__ pos, float4* __restrict__ vel,
                                  uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        pos[i] = aos[2 * (size_t)i];
        vel[i] = aos[2 * (size_t)i + 1];
    }
}

__global__ void soa_to_aos_kernel(const float4* __restrict__ pos, const float4* __restrict__ vel,
                                  float4* __restrict__ aos, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        aos[2 * (size_t)i] = pos[i];
        aos[2 * (size_t)i + 1] = vel[i];
    }
}

// Reads a buffer larger than L2 so the next step starts with none of its data cached.
__global__ void l2_flush_kernel(const float4* __restrict__ buf, size_t n4, float* sink) {
    float acc = 0.f;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n4; i += (size_t)gridDim.x * blockDim.x) {
        const float4 v = __ldcs(buf + i);
        acc += v.x + v.y + v.z + v.w;
    }
    if (acc == 1234567.0f) *sink = acc;  // never true for the zeroed buffer; keeps the loads
}

inline int grid_for(uint32_t n, int cap) {
    const uint32_t g = (n + 255u) / 256u;
    return (int)(g == 0 ? 1 : (g < (uint32_t)cap ? g : (uint32_t)cap));
}

}  // namespace

void launch_bin_count(const DevBuffers& d, const SceneConsts& sc, const LaunchDims& ld, cudaStream_t s) {
    int grid = grid_for(d.n, ld.grid_stream);
    const int need = (int)((d.num_tiles + 255u) / 256u);
    if (grid < need) grid = need;
    bin_count_kernel<false><<<grid, 256, 0, s>>>(d.pos_a, d.n, sc.bin, sc.R, BatchTables{}, d.keys, d.ranks, d.counts,
                                                 d.scan_desc, d.scan_tile_counter, d.num_tiles, d.err);
}

void launch_bin_count_batched(const DevBuffers& d, const BatchTables& bt, const LaunchDims& ld, cudaStream_t s) {
    int grid = grid_for(d.n, ld.grid_stream);
    const int need = (int)((d.num_tiles + 255u) / 256u);
    if (grid < need) grid = need;
    bin_count_kernel<true><<<grid, 256, 0, s>>>(d.pos_a, d.n, 0.f, 0, bt, d.keys, d.ranks, d.counts, d.scan_desc,
                                                d.scan_tile_counter, d.num_tiles, d.err);
}

void launch_scan_cells(const DevBuffers& d, cudaStream_t s) {
    scan_cells_kernel<<<d.num_tiles, SCAN_THREADS, 0, s>>>(d.counts, d.num_cells, d.start, d.cell_list,
                                                           d.num_nonempty, d.scan_desc, d.scan_tile_counter,
                                                           d.num_tiles, d.err);
}

void launch_scatter(const DevBuffers& d, const LaunchDims& ld, cudaStream_t s) {
    scatter_cells_kernel<<<grid_for(d.n, ld.grid_stream), 256, 0, s>>>(d.n, d.keys, d.ranks, d.start, d.unordered);
}

void launch_rank_gather(const DevBuffers& d, const LaunchDims& ld, cudaStream_t s, float* vxyz) {
    const int g = grid_for(d.n, ld.grid_stream);
    if (!d.vel_a)
        rank_gather_kernel<false, false><<<g, 256, 0, s>>>(d.n, d.keys, d.ranks, d.unordered, d.start, d.pos_a, nullptr,
                                                           nullptr, d.pos_b, nullptr, nullptr, d.perm, d.err, d.xyz,
                                                           d.xyz_stride, nullptr);
    else if (d.ids_a)
        rank_gather_kernel<true, true><<<g, 256, 0, s>>>(d.n, d.keys, d.ranks, d.unordered, d.start, d.pos_a, d.vel_a,
                                                         d.ids_a, d.pos_b, d.vel_b, d.ids_b, d.perm, d.err, d.xyz,
                                                         d.xyz_stride, vxyz);
    else
        rank_gather_kernel<false, true><<<g, 256, 0, s>>>(d.n, d.keys, d.ranks, d.unordered, d.start, d.pos_a,
                                                          d.vel_a, nullptr, d.pos_b, d.vel_b, nullptr, d.perm, d.err,
                                                          d.xyz, d.xyz_stride, vxyz);
}

void launch_aos_to_soa(const float4* aos, float4* pos, float4* vel, uint32_t n, cudaStream_t s) {
    aos_to_soa_kernel<<<grid_for(n, 1024), 256, 0, s>>>(aos, pos, vel, n);
}

void launch_soa_to_aos(const float4* pos, const float4* vel, float4* aos, uint32_t n, cudaStream_t s) {
    soa_to_aos_kernel<<<grid_for(n, 1024), 256, 0, s>>>(pos, vel, aos, n);
}

void launch_l2_flush(const float4* buf, size_t n4, float* sink, cudaStream_t s) {
    l2_flush_kernel<<<2048, 256, 0, s>>>(buf, n4, sink);
}

}  // namespace wc

extern "C" WC_API wc_status wc_debug_scan_stall(int on, uint32_t spin_limit) {
    wc::clear_error();
    const uint32_t stall = on ? 1u : 0u;
    const uint32_t limit = on ? spin_limit : wc::SCAN_SPIN_LIMIT;
    WC_CUDA_TRY(cudaMemcpyToSymbol(wc::g_scan_stall, &stall, sizeof stall));
    WC_CUDA_TRY(cudaMemcpyToSymbol(wc::g_scan_spin_limit, &limit, sizeof limit));
    return WC_OK;
}
