// wc_internal.h — device-side constants, buffer sets and stage launchers shared by the
// solver's translation units. Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/watercube.h"

namespace wc {

// Device error bits (OR-ed into DevBuffers::err by kernels; read at synchronisation points).
enum : uint32_t {
    DEVERR_NONFINITE = 1u << 0,    // a non-finite position was binned
    DEVERR_SCAN_TIMEOUT = 1u << 1,  // a scan tile gave up waiting on its predecessor
    DEVERR_MMA_TIMEOUT = 1u << 2,   // a tensor-core GEMM gave up waiting on its MMAs
    DEVERR_CELL_OVERFLOW = 1u << 3  // a cell held more than MAX_CELL_PARTICLES particles
};

// Cells holding more particles than this (256 times the rest density's ~8 per cell) are not
// evaluated: their particles get NaN density and keep their state, and the step reports
// WC_ERR_NUMERIC. Such a cell only arises from a collapsed or non-finite state (every NaN
// position bins to cell 0), where evaluating it would cost O(N^2) work per step.
constexpr uint32_t MAX_CELL_PARTICLES = 2048;
// The sort's stable in-cell rank counts, for each member of a cell, the members before it:
// O(k^2) per cell. Cells of more than this many particles (only reachable from a collapsed or
// non-finite state) take arrival order instead and are reported like an overfull cell.
constexpr uint32_t MAX_SORT_CELL_PARTICLES = 65536;

// Constants of one scene, by value in kernel parameters (single scene) or in a device table
// (batched scenes).
struct SceneConsts {
    float size, bin, h, h2, cull;  // cull: largest d2 with sqrtf(d2) < h
    float m, rho0, p0, k, mu;
    float c6, cs, cv;
    float max_speed, damping, border;
    float g[3];
    float mouse_o[3], mouse_d[3];
    int32_t R;
    uint32_t R_magic;  // ceil(2^32 / R) for R > 1 (division by R as a multiply-high), 0 for R = 1
    uint32_t eos, flags;
};

// Reciprocal for division by an invariant R > 1 (Granlund and Montgomery): m = ceil(2^32 / R).
inline uint32_t r_magic(uint32_t R) { return R > 1u ? (uint32_t)(((1ull << 32) + R - 1u) / R) : 0u; }

// q = n / R and n - q R for n < 2^31: the multiply-high estimate with m = ceil(2^32 / R) is the
// quotient or one more (its error n (m R - 2^32) / (R 2^32) is below 1), so one signed
// correction makes it exact.
__host__ __device__ __forceinline__ uint32_t div_R(uint32_t n, uint32_t R, uint32_t magic, uint32_t* rem) {
    if (R <= 1u) {
        *rem = 0u;
        return n;
    }
#ifdef __CUDA_ARCH__
    uint32_t q = __umulhi(n, magic);
#else
    uint32_t q = (uint32_t)(((uint64_t)n * magic) >> 32);
#endif
    int32_t r = (int32_t)(n - q * R);
    if (r < 0) {
        --q;
        r += (int32_t)R;
    }
    *rem = (uint32_t)r;
    return q;
}

#ifdef __CUDACC__
// The cell of a position: ivec3(p / binSize) clamped to [0, R-1] per axis (count.comp:31-33),
// IEEE division, NaN -> 0; the sort's binning, so any kernel recomputing a particle's cell from
// its (sorted) position finds the cell the sort put it in.
__device__ __forceinline__ int32_t bin_axis(float q, int32_t R) {
    if (!(q >= 1.0f)) return 0;
    if (q >= (float)(R - 1)) return R - 1;
    return (int32_t)q;
}
__device__ __forceinline__ uint32_t bin_key(float x, float y, float z, float bin, int32_t R, int32_t* cx, int32_t* cy,
                                            int32_t* cz) {
    *cx = bin_axis(__fdiv_rn(x, bin), R);
    *cy = bin_axis(__fdiv_rn(y, bin), R);
    *cz = bin_axis(__fdiv_rn(z, bin), R);
    return (uint32_t)((*cz * R + *cy) * R + *cx);
}
#endif

// Scene tables of a batch of independent scenes in one set of buffers (device memory). Scene s
// owns particle slots [poff[s], poff[s+1]) and cell keys [coff[s], coff[s] + R_s^3); one global
// counting sort over all keys therefore keeps every scene inside its own slot range.
constexpr uint32_t MAX_SCENES = 1024;
struct BatchTables {
    const SceneConsts* scenes;  // [num_scenes]
    const uint32_t* poff;       // [num_scenes + 1]
    const uint32_t* coff;       // [num_scenes + 1]
    uint32_t num_scenes;
};

// Largest s in [0, count) with offs[s] <= key, for ascending offs with offs[0] <= key.
__device__ __forceinline__ uint32_t find_scene(const uint32_t* offs, uint32_t count, uint32_t key) {
    uint32_t lo = 0, hi = count;
    while (hi - lo > 1u) {
        const uint32_t mid = (lo + hi) >> 1;
        if (offs[mid] <= key) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Per-step inputs that may change between steps without re-recording the step graph.
struct StepInputs {
    float dt;
    float g[3];
    float mouse_o[3], mouse_d[3];
    // A readback that overlaps the lane force pass (all null/zero otherwise): the pass also
    // writes every particle it stores as the host's AoS record into aos_out (two float4 per
    // slot), and the state's chunks of 32 slots form parts of part_chunks chunks; the warp that
    // finishes the last chunk of part r puts part_done[r] (device counters, zero between
    // launches) back to zero and writes seq to part_flag[r] (mapped host memory the host polls
    // before it copies the part out).
    float4* aos_out;
    uint32_t* part_done;
    uint32_t* part_flag;
    uint32_t part_chunks;
    uint32_t seq;
};

// Decoupled look-back scan over the cell histogram.
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 16;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;
constexpr uint32_t SCAN_SPIN_LIMIT = 1u << 22;  // ~0.3-1 s of polling before giving up

// SPH passes: 256-thread blocks of 8 cell teams (one warp each).
constexpr int SPH_THREADS = 256;
// Candidates a warp stages in shared memory per cell in the density pass (padding included).
constexpr int STAGE_CAP = 320;
// 32-bit words of neighbour bit strings per particle (density pass -> force pass): room for 4,096
// candidates, the 27-cell neighbourhoods of the 1M dam break's most compressed states (99th
// percentile 3,731 at step 1,750); a target with more tests its candidates again in the force pass.
constexpr int MASK_WORDS = 128;
// Force kernel dense path: per-lane neighbour list capacity ([CAP][32] words per warp).
constexpr int FORCE_LIST_CAP = 16;

// The stride of DevBuffers::xyz for n particles.
inline uint32_t xyz_stride_for(uint32_t n) { return ((n + 3u) & ~3u) + 4u; }

struct DevBuffers {
    uint32_t n;          // particles
    uint32_t num_cells;  // R^3
    uint32_t num_tiles;  // scan tiles
    // particle state: A = state buffer (particle_buffer1_), B = sorted buffer (particle_buffer2_)
    float4 *pos_a, *vel_a, *pos_b, *vel_b;
    uint32_t *ids_a, *ids_b;  // original indices (WC_FLAG_TRACK_IDS), else null
    // sort
    uint32_t *keys, *ranks, *unordered, *perm;
    uint32_t *counts;     // [C] histogram (zero between steps)
    uint32_t *start;      // [C+1] exclusive prefix + total
    uint32_t *cell_list;  // [C] non-empty cells, ascending
    // [0]: non-empty cells (written by the scan); [1], [2]: the density and force passes' cell
    // counters (dynamic scheduling; each launch leaves its counter at zero)
    uint32_t *num_nonempty;
    unsigned long long* scan_desc;  // [num_tiles]
    uint32_t* scan_tile_counter;
    uint32_t* ncount;  // [n] or null
    uint32_t* hits;    // [n * MASK_WORDS] neighbour bit strings
    // x, y, z of the sorted positions as three float arrays of xyz_stride (a multiple of 4 that
    // is >= n) elements each, written by the gather for the lane density pass's 16-byte loads of
    // four consecutive candidates; the padding past n is zero
    float* xyz;
    uint32_t xyz_stride;
    float4* accel;     // [n] acceleration of each particle in the last force pass, or null
    uint32_t* err;
};

// Neighbour pass variants (threads per cell): a 32-lane team per non-empty cell that splits the
// cell's targets into (targets x slices) and stages candidates in shared memory (PASSES_TEAM), or
// one lane per target walking its cell's 9 candidate rows (PASSES_LANE). The density pass of a
// variant writes its neighbour bit strings in the layout the force pass of the same variant
// reads; both variants select the same neighbour sets, their sums differ only in the order of
// the additions.
enum : int { PASSES_TEAM = 0, PASSES_LANE = 1 };

// Launch geometry computed once per handle.
struct LaunchDims {
    int sms;
    int grid_stream;   // blocks for the per-particle kernels
    int grid_density;  // persistent blocks
    int grid_force;
    int pass_variant;
};

LaunchDims compute_launch_dims(int device, int pass_variant = PASSES_LANE);

// The learned rollout's judge-step buffers of the force pass (sorted order): `out` receives
// (J, density rate) per particle, `rate` holds the density pass's (density rate, pressure rate).
struct FeatureBuffers {
    float4* out;
    const float2* rate;
};


// Stage launchers (wc_sort.cu, wc_sph.cu). All enqueue on `s` and never synchronise.
void launch_bin_count(const DevBuffers& d, const SceneConsts& sc, const LaunchDims& ld, cudaStream_t s);
void launch_scan_cells(const DevBuffers& d, cudaStream_t s);
void launch_scatter(const DevBuffers& d, const LaunchDims& ld, cudaStream_t s);
// vxyz (optional, the learned rollout's judge steps): also the sorted velocities' x, y, z as three
// arrays of d.xyz_stride elements.
void launch_rank_gather(const DevBuffers& d, const LaunchDims& ld, cudaStream_t s, float* vxyz = nullptr);
void launch_density(const DevBuffers& d, const SceneConsts& sc, const LaunchDims& ld, cudaStream_t s);
void launch_force(const DevBuffers& d, const SceneConsts& sc, const StepInputs& in, const LaunchDims& ld,
                  cudaStream_t s);
// Feature levels of the judge step's passes: FEAT_RATE (the stale mode's judge) — the density
// pass's judge sums and the force pass's own density rate; FEAT_FULL (the Taylor and network
// modes, and sample recording) — also the density and pressure rates from the density pass
// and the time derivative J of the acceleration from the force pass.
enum : int { FEAT_NONE = 0, FEAT_RATE = 1, FEAT_FULL = 2 };

// The learned rollout's judge step runs the lane passes with their feature outputs, whatever
// ld.pass_variant says: the density pass also writes rate[ti] = (density rate, pressure rate)
// from the gather's velocity arrays vxyz and, when judge_part is given, the judge's sums
// judge_part[m] = sum over the 32 slots of chunk m of |rho_carried / rho_SPH - 1| (rho_carried:
// the sorted buffer's .w before the pass); the force pass reads the neighbours' rates and writes
// feat[ti] = (J, density rate), J the time derivative of the SPH acceleration (sorted order).
void launch_density_feat(const DevBuffers& d, const SceneConsts& sc, const LaunchDims& ld, int level,
                         const float* vxyz, float2* rate, float* judge_part, cudaStream_t s);
void launch_density_batched_feat(const DevBuffers& d, const BatchTables& bt, const LaunchDims& ld, int level,
                                 const float* vxyz, float2* rate, float* judge_part, cudaStream_t s);
void launch_force_feat(const DevBuffers& d, const SceneConsts& sc, const StepInputs& in, const LaunchDims& ld,
                       int level, FeatureBuffers fb, cudaStream_t s);
void launch_force_batched_feat(const DevBuffers& d, const BatchTables& bt, const StepInputs& in, const LaunchDims& ld,
                               int level, FeatureBuffers fb, cudaStream_t s);
// AoS <-> SoA for host copies through a contiguous staging buffer.
void launch_aos_to_soa(const float4* aos, float4* pos, float4* vel, uint32_t n, cudaStream_t s);
void launch_soa_to_aos(const float4* pos, const float4* vel, float4* aos, uint32_t n, cudaStream_t s);
void launch_l2_flush(const float4* buf, size_t n4, float* sink, cudaStream_t s);

// A readback that overlaps the lane force pass (wc_fluid_update_host, wc_batch_step_host): the
// state's slots form READBACK_PARTS parts of whole chunks; the pass writes each stored particle's
// host record into the staging buffer and flags each finished part in mapped host memory
// (StepInputs readback fields); the host polls the flags in order and copies each part out on a
// second stream as it appears, so only the last part's copy follows the pass. No GPU-side wait.
constexpr uint32_t READBACK_PARTS = 8;
struct HostReadback {
    cudaStream_t copy_stream = nullptr;
    uint32_t* part_done = nullptr;      // device: finished chunks per part, zero between launches
    uint32_t* part_flag = nullptr;      // mapped host memory: the sequence number of the last
    uint32_t* part_flag_dev = nullptr;  // launch that finished each part, and its device address
    uint32_t seq = 0;
    uint32_t part_chunks = 0;
    uint32_t parts = 0;
    // Creates what is missing (on `s`) and sets the readback fields of `step` for n slots.
    wc_status arm(cudaStream_t s, uint32_t n, float4* staging, StepInputs& step);
    // After the pass is enqueued on `s`: copies the parts into out as they are flagged (or once
    // `s` has ended), then waits for the copies.
    wc_status drain(cudaStream_t s, uint32_t n, const float4* staging, wc_particle* out);
    void release();
};

// The same stages over a batch of scenes (wc_batch.cu): keys carry the scene's cell offset and
// every cell takes its scene's constants.
void launch_bin_count_batched(const DevBuffers& d, const BatchTables& bt, const LaunchDims& ld, cudaStream_t s);
void launch_density_batched(const DevBuffers& d, const BatchTables& bt, const LaunchDims& ld, cudaStream_t s);
void launch_force_batched(const DevBuffers& d, const BatchTables& bt, const StepInputs& in, const LaunchDims& ld,
                          cudaStream_t s);

// Host copies of the force kernel's arguments, in declaration order, so that a captured step
// graph's force node can be re-parameterised (dt, gravity, mouse ray) without re-capture.
struct ForceKernelArgs {
    SceneConsts sc;
    BatchTables bt;
    StepInputs in;
    uint32_t n;
    uint32_t num_cells;
    const float4* pos_b;
    const float4* vel_b;
    const uint32_t* ids_b;
    float4* pos_a;
    float4* vel_a;
    uint32_t* ids_a;
    const uint32_t* start;
    const uint32_t* cell_list;
    uint32_t* num_nonempty;
    const uint32_t* hits;
    float4* accel;
    uint32_t* err;
    FeatureBuffers feat{};  // the feature buffers of the learned rollout's judge steps (unused here)
    static constexpr int COUNT = 18;  // every parameter of force_lane_kernel, in order
    void* ptrs[COUNT];
    void bind() {
        void* p[COUNT] = {&sc,    &bt,    &in,    &n,     &num_cells, &pos_b,        &vel_b, &ids_b, &pos_a,
                          &vel_a, &ids_a, &start, &cell_list, &num_nonempty, &hits, &accel, &err, &feat};
        for (int i = 0; i < COUNT; ++i) ptrs[i] = p[i];
    }
};

// The kernel entry points the force node of a captured graph is recognised by.
const void* force_kernel_symbol(int pass_variant);
const void* force_kernel_batched_symbol(int pass_variant);
// Resident blocks per SM of the two neighbour passes (single-scene or batched variant).
void sph_occupancy(bool batched, int* density_blocks, int* force_blocks, int pass_variant);

// Internals of a wc_fluid, for the surrogate (wc_surrogate.cu), which works on a fluid's buffers.
struct FluidInternals {
    DevBuffers* d;
    const SceneConsts* sc;
    StepInputs* in;
    const wc_params* params;
    cudaStream_t stream;
};
FluidInternals fluid_internals(wc_fluid* f);

// A fluid or a batch of scenes as the learned rollout and its sample recorder drive them: the
// buffers, the constants (sc for a fluid; bt.num_scenes > 0 for a batch), the step inputs and
// the stream. Exactly one of fluid and batch is set.
struct StepTarget {
    DevBuffers* d;
    SceneConsts sc;
    BatchTables bt;
    StepInputs* in;
    LaunchDims ld;
    cudaStream_t stream;
    wc_fluid* fluid;
    wc_batch* batch;
};
StepTarget fluid_target(wc_fluid* f);
StepTarget batch_target(wc_batch* b);
wc_status batch_graph_step(wc_batch* b, float dt);  // one plain step (graph replay)
wc_status batch_check(wc_batch* b);                 // launch errors and device error word
wc_status fluid_check(wc_fluid* f);
// FP64 totals of a fluid's state buffer: mass, momentum x/y/z, kinetic and potential energy.
wc_status fluid_diagnostics(wc_fluid* f, double out[6]);
void fluid_enqueue_sort(wc_fluid* f);
wc_status fluid_graph_step(wc_fluid* f, float dt);  // one plain SPH step (graph replay)
void fluid_count_step(wc_fluid* f);
void fluid_set_step_count(wc_fluid* f, uint64_t steps);

SceneConsts make_scene_consts(const wc_params& p);
StepInputs make_step_inputs(const wc_params& p, float dt);

}  // namespace wc
