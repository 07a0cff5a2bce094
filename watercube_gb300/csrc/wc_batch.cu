// wc_batch.cu — many independent scenes advanced together (no counterpart in the reference).
//
// All scenes live in one set of buffers. Scene s owns particle slots [poff[s], poff[s+1]) and
// cell keys [coff[s], coff[s] + R_s^3): the bin kernel adds the scene's cell offset to the key it
// computes in the scene's own grid, so one global counting sort orders every scene at once and
// never moves a particle out of its scene's slots. The two neighbour passes look up each cell's
// scene (binary search in a shared-memory copy of the cell offsets) and use its constants. A
// step is the same six kernels as a single fluid, over all scenes, replayed as one CUDA graph.
//
// Also here: the autotuner (launch geometry and cell size, timed on graph replays), FP64
// per-scene diagnostics, and the scene draw of the 512-scene workload.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "wc_internal.h"
#include "wc_util.h"

using namespace wc;

namespace {

template <class T>
wc_status dalloc(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) return WC_OK;
    WC_TRY(::wc::device_alloc(reinterpret_cast<void**>(p), count * sizeof(T)));
    return WC_OK;
}

// FP64 reductions per scene: one block per scene, fixed-order tree, deterministic.
constexpr int DIAG_THREADS = 256;
__global__ void __launch_bounds__(DIAG_THREADS) scene_diag_kernel(const float4* __restrict__ pos,
                                                                  const float4* __restrict__ vel,
                                                                  const uint32_t* __restrict__ poff,
                                                                  const SceneConsts* __restrict__ scenes, float gx,
                                                                  float gy, float gz, double* __restrict__ out) {
    __shared__ double s_acc[5][DIAG_THREADS];
    const uint32_t s = blockIdx.x;
    const uint32_t b = poff[s], e = poff[s + 1];
    const double m = scenes[s].m;
    double a[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (uint32_t i = b + threadIdx.x; i < e; i += blockDim.x) {
        const float4 v = vel[i], p = pos[i];
        const double vx = v.x, vy = v.y, vz = v.z;
        a[0] += m * vx;
        a[1] += m * vy;
        a[2] += m * vz;
        a[3] += 0.5 * m * (vx * vx + vy * vy + vz * vz);
        a[4] -= m * ((double)gx * p.x + (double)gy * p.y + (double)gz * p.z);
    }
    for (int q = 0; q < 5; ++q) s_acc[q][threadIdx.x] = a[q];
    __syncthreads();
    for (int half = DIAG_THREADS / 2; half > 0; half >>= 1) {
        if ((int)threadIdx.x < half)
            for (int q = 0; q < 5; ++q) s_acc[q][threadIdx.x] += s_acc[q][threadIdx.x + half];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[6 * s + 0] = m * (double)(e - b);
        for (int q = 0; q < 5; ++q) out[6 * s + 1 + q] = s_acc[q][0];
    }
}

inline uint64_t splitmix64(uint64_t& state) {
    uint64_t z = (state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
inline double unit53(uint64_t& st) { return (double)(splitmix64(st) >> 11) * (1.0 / 9007199254740992.0); }
// Box-Muller; two uniforms per normal (the second of each pair is discarded for simplicity).
inline double normal(uint64_t& st) {
    double u1 = unit53(st), u2 = unit53(st);
    if (u1 < 1e-300) u1 = 1e-300;
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
}

struct TuneKey {
    uint64_t n;
    uint64_t cells;
    bool operator<(const TuneKey& o) const { return n < o.n || (n == o.n && cells < o.cells); }
};
std::mutex g_tune_mutex;
std::map<TuneKey, wc_tuning> g_tune_cache;

}  // namespace

struct wc_batch {
    std::vector<wc_params> base;  // the caller's parameters, finalized
    std::vector<wc_params> params;  // with the grid of the current cell factor
    std::vector<uint32_t> poff, coff;
    uint32_t S = 0;
    uint64_t n = 0;
    uint64_t cells_cap = 0;
    SceneConsts* d_scenes = nullptr;
    uint32_t* d_poff = nullptr;
    uint32_t* d_coff = nullptr;
    double* d_diag = nullptr;
    DevBuffers d{};
    LaunchDims ld{};
    int device = 0;
    int max_density_blocks = 1, max_force_blocks = 1;
    cudaStream_t stream = nullptr;
    StepInputs in{};
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphNode_t force_node = nullptr;
    cudaKernelNodeParams force_params{};
    ForceKernelArgs fargs{};
    StepInputs graph_in{};
    float4* staging = nullptr;
    uint32_t* h_err = nullptr;
    HostReadback readback{};  // wc_batch_step_host
    float4* flush_buf = nullptr;
    size_t flush_n4 = 0;
    float* flush_sink = nullptr;
    wc_tuning tuning{};
    bool setup_done = false;
};

namespace {

BatchTables tables(const wc_batch* b) { return BatchTables{b->d_scenes, b->d_poff, b->d_coff, b->S}; }

void drop_graph(wc_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    b->force_node = nullptr;
}

void free_batch(wc_batch* b) {
    drop_graph(b);
    DevBuffers& d = b->d;
    void* ptrs[] = {d.pos_a,     d.vel_a,        d.pos_b,      d.vel_b,  d.keys,         d.ranks,
                    d.unordered, d.perm,         d.counts,     d.start,  d.cell_list,    d.num_nonempty,
                    d.scan_desc, d.scan_tile_counter, d.err,   d.hits,   b->d_scenes,    b->d_poff,
                    b->d_coff,   b->d_diag,      b->staging,   b->flush_buf, b->flush_sink, d.ids_a,
                    d.ids_b,     d.accel,        d.xyz};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (b->h_err) cudaFreeHost(b->h_err);
    b->readback.release();
    if (b->stream) cudaStreamDestroy(b->stream);
}

uint32_t grid_for_factor(const wc_params& p, float factor) {
    const float r = std::floor(p.size / (p.kernel_radius * factor));
    return r < 1.0f ? 1u : (r > 1024.0f ? 1024u : (uint32_t)r);
}

// Scene grids and cell offsets for a cell edge of factor * h (factor >= 1 keeps the 27-cell
// search exact); uploads the tables.
wc_status apply_cell_factor(wc_batch* b, float factor) {
    b->params = b->base;
    b->coff.assign(b->S + 1, 0);
    std::vector<SceneConsts> sc(b->S);
    uint64_t c = 0;
    for (uint32_t s = 0; s < b->S; ++s) {
        wc_params& p = b->params[s];
        p.grid_res = grid_for_factor(b->base[s], factor);
        p.bin_size = p.size / (float)p.grid_res;
        sc[s] = make_scene_consts(p);
        b->coff[s] = (uint32_t)c;
        c += (uint64_t)p.grid_res * p.grid_res * p.grid_res;
    }
    if (c > b->cells_cap) return fail(WC_ERR_INVALID_ARG, "cell factor %g needs %llu cells, capacity %llu", factor,
                                      (unsigned long long)c, (unsigned long long)b->cells_cap);
    b->coff[b->S] = (uint32_t)c;
    b->d.num_cells = (uint32_t)c;
    b->d.num_tiles = (uint32_t)((c + SCAN_TILE - 1) / SCAN_TILE);
    WC_CUDA_TRY(cudaMemcpyAsync(b->d_scenes, sc.data(), sizeof(SceneConsts) * b->S, cudaMemcpyHostToDevice, b->stream));
    WC_CUDA_TRY(cudaMemcpyAsync(b->d_coff, b->coff.data(), sizeof(uint32_t) * (b->S + 1), cudaMemcpyHostToDevice,
                                b->stream));
    WC_CUDA_TRY(cudaMemsetAsync(b->d.counts, 0, sizeof(uint32_t) * b->cells_cap, b->stream));
    WC_CUDA_TRY(cudaStreamSynchronize(b->stream));
    b->tuning.cell_factor = factor;
    drop_graph(b);
    return WC_OK;
}

void apply_geometry(wc_batch* b, const wc_tuning& t) {
    const int variant = t.pass_variant == WC_PASSES_TEAM ? PASSES_TEAM : PASSES_LANE;
    if (variant != b->ld.pass_variant) {
        b->ld.pass_variant = variant;
        sph_occupancy(true, &b->max_density_blocks, &b->max_force_blocks, variant);
    }
    b->tuning.pass_variant = (uint32_t)variant;
    b->ld.grid_density = b->ld.sms * (int)std::max(1u, std::min(t.density_blocks_per_sm, (uint32_t)b->max_density_blocks));
    b->ld.grid_force = b->ld.sms * (int)std::max(1u, std::min(t.force_blocks_per_sm, (uint32_t)b->max_force_blocks));
    b->ld.grid_stream = b->ld.sms * (int)std::max(1u, t.stream_blocks_per_sm);
    b->tuning.density_blocks_per_sm = (uint32_t)(b->ld.grid_density / b->ld.sms);
    b->tuning.force_blocks_per_sm = (uint32_t)(b->ld.grid_force / b->ld.sms);
    b->tuning.stream_blocks_per_sm = (uint32_t)(b->ld.grid_stream / b->ld.sms);
    drop_graph(b);
}

void enqueue_step(wc_batch* b, const StepInputs& in) {
    const BatchTables bt = tables(b);
    launch_bin_count_batched(b->d, bt, b->ld, b->stream);
    launch_scan_cells(b->d, b->stream);
    launch_scatter(b->d, b->ld, b->stream);
    launch_rank_gather(b->d, b->ld, b->stream);
    launch_density_batched(b->d, bt, b->ld, b->stream);
    launch_force_batched(b->d, bt, in, b->ld, b->stream);
}

wc_status capture(wc_batch* b, const StepInputs& in) {
    WC_CUDA_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    enqueue_step(b, in);
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
    if (ce != cudaSuccess) return fail(WC_ERR_CUDA, "batch graph capture failed: %s", cudaGetErrorString(ce));
    b->graph = g;
    WC_CUDA_TRY(cudaGraphInstantiate(&b->exec, g, 0));
    size_t count = 0;
    WC_CUDA_TRY(cudaGraphGetNodes(g, nullptr, &count));
    std::vector<cudaGraphNode_t> nodes(count);
    WC_CUDA_TRY(cudaGraphGetNodes(g, nodes.data(), &count));
    for (cudaGraphNode_t nd : nodes) {
        cudaGraphNodeType ty;
        WC_CUDA_TRY(cudaGraphNodeGetType(nd, &ty));
        if (ty != cudaGraphNodeTypeKernel) continue;
        cudaKernelNodeParams kp;
        WC_CUDA_TRY(cudaGraphKernelNodeGetParams(nd, &kp));
        if (kp.func == force_kernel_batched_symbol(b->ld.pass_variant)) {
            b->force_node = nd;
            b->force_params = kp;
        }
    }
    if (!b->force_node) return fail(WC_ERR_CUDA, "batch graph has no force node");
    ForceKernelArgs& a = b->fargs;
    a.sc = SceneConsts{};
    a.bt = tables(b);
    a.in = in;
    a.n = b->d.n;
    a.num_cells = b->d.num_cells;
    a.pos_b = b->d.pos_b;
    a.vel_b = b->d.vel_b;
    a.ids_b = b->d.ids_b;
    a.pos_a = b->d.pos_a;
    a.vel_a = b->d.vel_a;
    a.ids_a = b->d.ids_a;
    a.start = b->d.start;
    a.cell_list = b->d.cell_list;
    a.num_nonempty = b->d.num_nonempty;
    a.hits = b->d.hits;
    a.accel = b->d.accel;
    a.err = b->d.err;
    a.bind();
    b->graph_in = in;
    return WC_OK;
}

wc_status launch(wc_batch* b, const StepInputs& in) {
    if (!b->exec) {
        WC_TRY(capture(b, in));
    } else if (std::memcmp(&in, &b->graph_in, sizeof in) != 0) {
        b->fargs.in = in;
        cudaKernelNodeParams kp = b->force_params;
        kp.kernelParams = b->fargs.ptrs;
        kp.extra = nullptr;
        WC_CUDA_TRY(cudaGraphExecKernelNodeSetParams(b->exec, b->force_node, &kp));
        b->graph_in = in;
    }
    WC_CUDA_TRY(cudaGraphLaunch(b->exec, b->stream));
    return WC_OK;
}

wc_status read_errors(wc_batch* b) {
    WC_CUDA_TRY(cudaStreamSynchronize(b->stream));
    WC_CUDA_TRY(cudaMemcpyAsync(b->h_err, b->d.err, sizeof(uint32_t), cudaMemcpyDeviceToHost, b->stream));
    WC_CUDA_TRY(cudaStreamSynchronize(b->stream));
    const uint32_t e = *b->h_err;
    if (e) {
        WC_CUDA_TRY(cudaMemsetAsync(b->d.err, 0, sizeof(uint32_t), b->stream));
        WC_CUDA_TRY(cudaStreamSynchronize(b->stream));
        if (e & DEVERR_SCAN_TIMEOUT) return fail(WC_ERR_TIMEOUT, "cell scan look-back exceeded its wait limit");
        if (e & DEVERR_CELL_OVERFLOW)
            return fail(WC_ERR_NUMERIC, "a cell held more than %u particles (a collapsed or non-finite state); its "
                                        "particles were not evaluated", MAX_CELL_PARTICLES);
        return fail(WC_ERR_NUMERIC, "a particle position was NaN or infinite when it was binned");
    }
    return WC_OK;
}

wc_status ensure_staging(wc_batch* b) {
    if (!b->staging && b->n) WC_TRY(dalloc(&b->staging, 2 * (size_t)b->n));
    return WC_OK;
}

wc_status require(const wc_batch* b, bool need_setup) {
    if (!b) return fail(WC_ERR_INVALID_ARG, "null batch handle");
    if (need_setup && !b->setup_done) return fail(WC_ERR_STATE, "wc_batch_setup has not been called");
    return WC_OK;
}

// Mean device time of `steps` graph replays after `warm` untimed ones.
wc_status time_replays(wc_batch* b, const StepInputs& in, int warm, int steps, float* ms) {
    for (int i = 0; i < warm; ++i) WC_TRY(launch(b, in));
    cudaEvent_t e0, e1;
    WC_CUDA_TRY(cudaEventCreate(&e0));
    WC_CUDA_TRY(cudaEventCreate(&e1));
    cudaEventRecord(e0, b->stream);
    wc_status st = WC_OK;
    for (int i = 0; i < steps && st == WC_OK; ++i) st = launch(b, in);
    cudaEventRecord(e1, b->stream);
    if (st == WC_OK) st = read_errors(b);
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *ms = t / (float)steps;
    return st;
}

wc_status save_state(wc_batch* b) {
    WC_TRY(ensure_staging(b));
    WC_CUDA_TRY(cudaMemcpyAsync(b->staging, b->d.pos_a, sizeof(float4) * b->n, cudaMemcpyDeviceToDevice, b->stream));
    WC_CUDA_TRY(cudaMemcpyAsync(b->staging + b->n, b->d.vel_a, sizeof(float4) * b->n, cudaMemcpyDeviceToDevice,
                                b->stream));
    return WC_OK;
}

wc_status restore_state(wc_batch* b) {
    WC_CUDA_TRY(cudaMemcpyAsync(b->d.pos_a, b->staging, sizeof(float4) * b->n, cudaMemcpyDeviceToDevice, b->stream));
    WC_CUDA_TRY(cudaMemcpyAsync(b->d.vel_a, b->staging + b->n, sizeof(float4) * b->n, cudaMemcpyDeviceToDevice,
                                b->stream));
    return WC_OK;
}

std::string cache_path() {
    const char* p = std::getenv("WC_TUNE_CACHE");
    return p ? std::string(p) : std::string();
}

bool cache_lookup(const TuneKey& k, wc_tuning* out) {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    auto it = g_tune_cache.find(k);
    if (it != g_tune_cache.end()) {
        *out = it->second;
        return true;
    }
    const std::string path = cache_path();
    if (path.empty()) return false;
    FILE* f = std::fopen(path.c_str(), "r");
    if (!f) return false;
    unsigned long long n, c;
    unsigned d, fo, st, fv;
    float cf, ms;
    bool found = false;
    while (std::fscanf(f, "%llu %llu %u %u %u %f %f %u", &n, &c, &d, &fo, &st, &cf, &ms, &fv) == 8) {
        if (n == k.n && c == k.cells) {
            *out = wc_tuning{d, fo, st, cf, ms, 0, fv};
            found = true;
        }
    }
    std::fclose(f);
    if (found) g_tune_cache[k] = *out;
    return found;
}

void cache_store(const TuneKey& k, const wc_tuning& t) {
    std::lock_guard<std::mutex> lock(g_tune_mutex);
    g_tune_cache[k] = t;
    const std::string path = cache_path();
    if (path.empty()) return;
    FILE* f = std::fopen(path.c_str(), "a");
    if (!f) return;
    std::fprintf(f, "%llu %llu %u %u %u %.3f %.6f %u\n", (unsigned long long)k.n, (unsigned long long)k.cells,
                 t.density_blocks_per_sm, t.force_blocks_per_sm, t.stream_blocks_per_sm, t.cell_factor, t.step_ms,
                 t.pass_variant);
    std::fclose(f);
}

}  // namespace

namespace wc {

StepTarget batch_target(wc_batch* b) {
    StepTarget t{};
    t.d = &b->d;
    t.bt = tables(b);
    t.in = &b->in;
    t.ld = b->ld;
    t.stream = b->stream;
    t.batch = b;
    return t;
}

wc_status batch_graph_step(wc_batch* b, float dt) {
    b->in.dt = dt;
    return launch(b, b->in);
}

wc_status batch_check(wc_batch* b) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(WC_ERR_CUDA, "kernel launch failed: %s", cudaGetErrorString(e));
    return read_errors(b);
}

}  // namespace wc

extern "C" {

WC_API wc_status wc_generate_batch_specs(uint64_t seed, uint32_t num_scenes, uint32_t n_min, uint32_t n_max,
                                         wc_scene_spec* out) {
    clear_error();
    if (!out && num_scenes) return fail(WC_ERR_INVALID_ARG, "null output");
    if (n_min == 0 || n_max < n_min) return fail(WC_ERR_INVALID_ARG, "bad particle count range");
    uint64_t st = seed;
    const double lo = std::log((double)n_min), hi = std::log((double)n_max);
    for (uint32_t s = 0; s < num_scenes; ++s) {
        wc_scene_spec& sp = out[s];
        std::memset(&sp, 0, sizeof sp);
        const double ln = lo + (hi - lo) * unit53(st);
        sp.num_particles = (uint32_t)std::min<double>(n_max, std::max<double>(n_min, std::floor(std::exp(ln) + 0.5)));
        for (int a = 0; a < 3; ++a) {
            const float side = (float)(0.2 + 0.5 * unit53(st));
            const float off = a == 1 ? 0.0f : (float)((1.0 - side) * unit53(st));
            sp.block_min[a] = off;
            sp.block_max[a] = off + side;
        }
        sp.stiffness = (float)(2.0 + 4.0 * unit53(st));
        sp.velocity_sigma = 0.5f;
        sp.seed = splitmix64(st);
    }
    return WC_OK;
}

WC_API wc_status wc_scene_params(const wc_scene_spec* spec, wc_params* out) {
    clear_error();
    if (!spec || !out) return fail(WC_ERR_INVALID_ARG, "null argument");
    if (spec->num_particles == 0) return fail(WC_ERR_INVALID_ARG, "scene without particles");
    double vol = 1.0;
    for (int a = 0; a < 3; ++a) vol *= (double)spec->block_max[a] - (double)spec->block_min[a];
    if (!(vol > 0.0)) return fail(WC_ERR_INVALID_ARG, "empty scene block");
    wc_params_dam_break(out, spec->num_particles);
    const double s = std::cbrt(vol / (double)spec->num_particles);
    out->kernel_radius = (float)(2.0 * s);
    out->particle_radius = (float)(0.5 * s);
    out->particle_mass = (float)((double)out->rest_density * s * s * s);
    out->stiffness = spec->stiffness;
    out->grid_res = 0;
    return wc_params_finalize(out);
}

WC_API wc_status wc_generate_scene(const wc_scene_spec* spec, const wc_params* p, wc_particle* out) {
    clear_error();
    if (!spec || !p || (!out && spec->num_particles)) return fail(WC_ERR_INVALID_ARG, "null argument");
    const double s = 0.5 * (double)p->kernel_radius;
    uint32_t dims[3];
    for (int a = 0; a < 3; ++a) {
        const double side = (double)spec->block_max[a] - (double)spec->block_min[a];
        dims[a] = std::max(1u, (uint32_t)std::floor(side / s));
    }
    // Enough sites for every particle: grow the y extent (the block becomes taller if needed).
    while ((uint64_t)dims[0] * dims[1] * dims[2] < spec->num_particles) ++dims[1];
    uint64_t st = spec->seed;
    const float js = 0.01f * p->kernel_radius;
    for (uint32_t q = 0; q < spec->num_particles; ++q) {
        const uint32_t i = q % dims[0], k = (q / dims[0]) % dims[2], j = q / (dims[0] * dims[2]);
        const double lat[3] = {spec->block_min[0] + (i + 0.5) * s, spec->block_min[1] + (j + 0.5) * s,
                               spec->block_min[2] + (k + 0.5) * s};
        wc_particle& o = out[q];
        for (int a = 0; a < 3; ++a) {
            const float u = (float)(splitmix64(st) >> 40) * (1.0f / 16777216.0f);
            o.position[a] = (float)lat[a] + (2.0f * u - 1.0f) * js;
        }
        for (int a = 0; a < 3; ++a) o.velocity[a] = (float)(spec->velocity_sigma * normal(st));
        o.density = 0.0f;
        o.pressure = 0.0f;
    }
    return WC_OK;
}

WC_API wc_status wc_batch_create(const wc_params* scenes, uint32_t num_scenes, wc_batch** out) {
    clear_error();
    if (!scenes || !out || num_scenes == 0) return fail(WC_ERR_INVALID_ARG, "wc_batch_create: no scenes");
    if (num_scenes > MAX_SCENES) return fail(WC_ERR_INVALID_ARG, "at most %u scenes per batch", MAX_SCENES);
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(WC_ERR_CUDA, "no CUDA device");
    wc_batch* b = new (std::nothrow) wc_batch();
    if (!b) return fail(WC_ERR_OOM, "host allocation failed");
    b->S = num_scenes;
    b->base.assign(scenes, scenes + num_scenes);
    b->poff.assign(num_scenes + 1, 0);
    uint64_t n = 0, cells = 0;
    wc_status st = WC_OK;
    for (uint32_t s = 0; s < num_scenes && st == WC_OK; ++s) {
        wc_params& p = b->base[s];
        st = wc_params_finalize(&p);
        p.flags &= ~(uint32_t)(WC_FLAG_TRACK_IDS | WC_FLAG_NEIGHBOR_COUNTS);
        b->poff[s] = (uint32_t)n;
        n += p.num_particles;
        const uint64_t r = grid_for_factor(p, 1.0f);
        cells += r * r * r;
    }
    if (st == WC_OK && (n >= (1ull << 31) || cells >= (1ull << 31)))
        st = fail(WC_ERR_INVALID_ARG, "batch too large: %llu particles, %llu cells", (unsigned long long)n,
                  (unsigned long long)cells);
    if (st != WC_OK) {
        delete b;
        return st;
    }
    b->poff[num_scenes] = (uint32_t)n;
    b->n = n;
    b->cells_cap = cells;
    cudaGetDevice(&b->device);
    DevBuffers& d = b->d;
    d.n = (uint32_t)n;
    const size_t tiles_cap = (cells + SCAN_TILE - 1) / SCAN_TILE;
    st = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) == cudaSuccess
             ? WC_OK
             : fail(WC_ERR_CUDA, "stream creation failed");
    if (st == WC_OK) st = dalloc(&d.pos_a, n);
    if (st == WC_OK) st = dalloc(&d.vel_a, n);
    if (st == WC_OK) st = dalloc(&d.pos_b, n);
    if (st == WC_OK) st = dalloc(&d.vel_b, n);
    if (st == WC_OK) st = dalloc(&d.keys, n);
    if (st == WC_OK) st = dalloc(&d.ranks, n);
    if (st == WC_OK) st = dalloc(&d.unordered, n);
    if (st == WC_OK) st = dalloc(&d.perm, n);
    if (st == WC_OK) st = dalloc(&d.ids_a, n);
    if (st == WC_OK) st = dalloc(&d.ids_b, n);
    if (st == WC_OK) st = dalloc(&d.hits, (size_t)n * MASK_WORDS);
    d.xyz_stride = xyz_stride_for((uint32_t)n);
    if (st == WC_OK) st = dalloc(&d.xyz, 3 * (size_t)d.xyz_stride);
    if (st == WC_OK) st = dalloc(&d.counts, cells);
    if (st == WC_OK) st = dalloc(&d.start, cells + 1);
    if (st == WC_OK) st = dalloc(&d.cell_list, cells);
    if (st == WC_OK) st = dalloc(&d.num_nonempty, 3);
    if (st == WC_OK) st = dalloc(&d.scan_desc, tiles_cap);
    if (st == WC_OK) st = dalloc(&d.scan_tile_counter, 1);
    if (st == WC_OK) st = dalloc(&d.err, 1);
    if (st == WC_OK) st = dalloc(&b->d_scenes, num_scenes);
    if (st == WC_OK) st = dalloc(&b->d_poff, num_scenes + 1);
    if (st == WC_OK) st = dalloc(&b->d_coff, num_scenes + 1);
    if (st == WC_OK) st = dalloc(&b->d_diag, 6 * (size_t)num_scenes);
    if (st == WC_OK && cudaMallocHost(reinterpret_cast<void**>(&b->h_err), sizeof(uint32_t)) != cudaSuccess)
        st = fail(WC_ERR_OOM, "pinned allocation failed");
    if (st == WC_OK && cudaMemcpyAsync(b->d_poff, b->poff.data(), sizeof(uint32_t) * (num_scenes + 1),
                                       cudaMemcpyHostToDevice, b->stream) != cudaSuccess)
        st = fail(WC_ERR_CUDA, "table upload failed");
    if (st == WC_OK) {
        cudaMemsetAsync(d.err, 0, sizeof(uint32_t), b->stream);
        cudaMemsetAsync(d.num_nonempty, 0, 3 * sizeof(uint32_t), b->stream);
        cudaMemsetAsync(d.start, 0, sizeof(uint32_t) * (cells + 1), b->stream);
        if (n) cudaMemsetAsync(d.hits, 0, sizeof(uint32_t) * MASK_WORDS * (size_t)n, b->stream);
        cudaMemsetAsync(d.xyz, 0, sizeof(float) * 3 * (size_t)d.xyz_stride, b->stream);
        // the force pass variant of the scenes' flags (a fluid with the same flags gives each scene's
        // result bit for bit)
        const int variant = (b->base[0].flags & WC_FLAG_CELL_TEAMS) ? PASSES_TEAM : PASSES_LANE;
        b->ld = compute_launch_dims(b->device, variant);
        sph_occupancy(true, &b->max_density_blocks, &b->max_force_blocks, variant);
        b->ld.grid_density = b->ld.sms * b->max_density_blocks;
        b->ld.grid_force = b->ld.sms * b->max_force_blocks;
        b->tuning = wc_tuning{(uint32_t)b->max_density_blocks, (uint32_t)b->max_force_blocks, 8u, 1.0f, 0.f, 0u,
                              (uint32_t)variant};
        b->in = make_step_inputs(b->base[0], 0.0f);
        st = apply_cell_factor(b, 1.0f);
    }
    if (st != WC_OK) {
        free_batch(b);
        delete b;
        return st;
    }
    *out = b;
    return WC_OK;
}

WC_API void wc_batch_destroy(wc_batch* b) {
    if (!b) return;
    if (b->stream) cudaStreamSynchronize(b->stream);
    free_batch(b);
    delete b;
}

WC_API wc_status wc_batch_set_particles(wc_batch* b, const wc_particle* in, uint64_t total) {
    clear_error();
    WC_NVTX("wc_batch_set_particles");
    WC_TRY(require(b, false));
    if (total != b->n) return fail(WC_ERR_INVALID_ARG, "%llu particles given, batch holds %llu",
                                   (unsigned long long)total, (unsigned long long)b->n);
    if (!total) return WC_OK;
    if (!in) return fail(WC_ERR_INVALID_ARG, "null input");
    WC_TRY(ensure_staging(b));
    WC_CUDA_TRY(cudaMemcpyAsync(b->staging, in, sizeof(wc_particle) * total, cudaMemcpyHostToDevice, b->stream));
    launch_aos_to_soa(b->staging, b->d.pos_a, b->d.vel_a, (uint32_t)total, b->stream);
    WC_CUDA_TRY(cudaStreamSynchronize(b->stream));
    return WC_OK;
}

WC_API wc_status wc_batch_setup(wc_batch* b, const wc_particle* initial, uint64_t total) {
    WC_TRY(wc_batch_set_particles(b, initial, total));
    if (b->n) {
        std::vector<uint32_t> iota(b->n);
        for (uint64_t i = 0; i < b->n; ++i) iota[i] = (uint32_t)i;
        WC_CUDA_TRY(cudaMemcpyAsync(b->d.ids_a, iota.data(), sizeof(uint32_t) * b->n, cudaMemcpyHostToDevice, b->stream));
        WC_CUDA_TRY(cudaStreamSynchronize(b->stream));
    }
    b->setup_done = true;
    return WC_OK;
}

WC_API wc_status wc_batch_set_recording(wc_batch* b, int on) {
    clear_error();
    WC_NVTX("wc_batch_setup");
    WC_TRY(require(b, false));
    if (on && !b->d.accel) {
        WC_TRY(dalloc(&b->d.accel, b->n));
        if (b->n) WC_CUDA_TRY(cudaMemsetAsync(b->d.accel, 0, sizeof(float4) * b->n, b->stream));
    } else if (!on && b->d.accel) {
        WC_CUDA_TRY(cudaStreamSynchronize(b->stream));
        cudaFree(b->d.accel);
        b->d.accel = nullptr;
    }
    drop_graph(b);
    return WC_OK;
}

WC_API wc_status wc_batch_get_accelerations(wc_batch* b, float* out, uint64_t total) {
    clear_error();
    WC_TRY(require(b, false));
    if (!b->d.accel) return fail(WC_ERR_STATE, "recording is off (wc_batch_set_recording)");
    if (total != b->n || (!out && total)) return fail(WC_ERR_INVALID_ARG, "bad acceleration buffer");
    if (total) WC_CUDA_TRY(cudaMemcpyAsync(out, b->d.accel, sizeof(float4) * total, cudaMemcpyDeviceToHost, b->stream));
    return read_errors(b);
}

WC_API wc_status wc_batch_get_ids(wc_batch* b, uint32_t* out, uint64_t total) {
    clear_error();
    WC_TRY(require(b, false));
    if (total != b->n || (!out && total)) return fail(WC_ERR_INVALID_ARG, "bad id buffer");
    if (total) WC_CUDA_TRY(cudaMemcpyAsync(out, b->d.ids_a, sizeof(uint32_t) * total, cudaMemcpyDeviceToHost, b->stream));
    return read_errors(b);
}

WC_API wc_status wc_batch_get_particles(wc_batch* b, wc_particle* out, uint64_t total) {
    clear_error();
    WC_NVTX("wc_batch_get_particles");
    WC_TRY(require(b, false));
    if (total != b->n) return fail(WC_ERR_INVALID_ARG, "%llu particles asked, batch holds %llu",
                                   (unsigned long long)total, (unsigned long long)b->n);
    if (!total) return read_errors(b);
    if (!out) return fail(WC_ERR_INVALID_ARG, "null output");
    WC_TRY(ensure_staging(b));
    launch_soa_to_aos(b->d.pos_a, b->d.vel_a, b->staging, (uint32_t)total, b->stream);
    WC_CUDA_TRY(cudaMemcpyAsync(out, b->staging, sizeof(wc_particle) * total, cudaMemcpyDeviceToHost, b->stream));
    return read_errors(b);
}

WC_API wc_status wc_batch_step_host(wc_batch* b, float dt, const wc_particle* in, wc_particle* out, uint64_t total) {
    clear_error();
    WC_NVTX("wc_batch_step_host");
    WC_TRY(require(b, true));
    if (total != b->n) return fail(WC_ERR_INVALID_ARG, "%llu particles given, batch holds %llu",
                                   (unsigned long long)total, (unsigned long long)b->n);
    if (!total || !out || b->ld.pass_variant != PASSES_LANE) {
        // nothing to overlap: the three calls in turn
        if (total && in) WC_TRY(wc_batch_set_particles(b, in, total));
        WC_TRY(wc_batch_step(b, dt, 1));
        return out ? wc_batch_get_particles(b, out, total) : WC_OK;
    }
    const uint32_t n = (uint32_t)total;
    b->in.dt = dt;
    WC_TRY(ensure_staging(b));
    if (in) {
        // the final wait covers the copy from in
        WC_CUDA_TRY(cudaMemcpyAsync(b->staging, in, sizeof(wc_particle) * total, cudaMemcpyHostToDevice, b->stream));
        launch_aos_to_soa(b->staging, b->d.pos_a, b->d.vel_a, n, b->stream);
    }
    StepInputs step = b->in;
    WC_TRY(b->readback.arm(b->stream, n, b->staging, step));
    enqueue_step(b, step);  // the graph's stages, launched directly with the readback fields
    WC_CUDA_TRY(cudaGetLastError());
    WC_TRY(b->readback.drain(b->stream, n, b->staging, out));
    return read_errors(b);
}

WC_API wc_status wc_batch_step(wc_batch* b, float dt, uint32_t nsteps) {
    clear_error();
    WC_NVTX("wc_batch_step");
    WC_TRY(require(b, true));
    b->in.dt = dt;
    for (uint32_t s = 0; s < nsteps; ++s) WC_TRY(launch(b, b->in));
    return WC_OK;
}

WC_API wc_status wc_batch_scene_offsets(const wc_batch* b, uint64_t* offsets) {
    clear_error();
    WC_TRY(require(b, false));
    if (!offsets) return fail(WC_ERR_INVALID_ARG, "null output");
    for (uint32_t s = 0; s <= b->S; ++s) offsets[s] = b->poff[s];
    return WC_OK;
}

WC_API uint32_t wc_batch_num_scenes(const wc_batch* b) { return b ? b->S : 0; }
WC_API uint64_t wc_batch_num_particles(const wc_batch* b) { return b ? b->n : 0; }

WC_API wc_status wc_batch_diagnostics(wc_batch* b, double* out) {
    clear_error();
    WC_TRY(require(b, false));
    if (!out) return fail(WC_ERR_INVALID_ARG, "null output");
    scene_diag_kernel<<<b->S, DIAG_THREADS, 0, b->stream>>>(b->d.pos_a, b->d.vel_a, b->d_poff, b->d_scenes,
                                                              b->in.g[0], b->in.g[1], b->in.g[2], b->d_diag);
    WC_CUDA_TRY(cudaGetLastError());
    WC_CUDA_TRY(cudaMemcpyAsync(out, b->d_diag, sizeof(double) * 6 * b->S, cudaMemcpyDeviceToHost, b->stream));
    return read_errors(b);
}

WC_API wc_status wc_batch_time_steps(wc_batch* b, float dt, uint32_t nsteps, int flush_l2, float* step_ms) {
    clear_error();
    WC_NVTX("wc_batch_time_steps");
    WC_TRY(require(b, true));
    if (!step_ms && nsteps) return fail(WC_ERR_INVALID_ARG, "null step_ms");
    if (flush_l2 && !b->flush_buf) {
        int l2 = 0;
        cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, b->device);
        const size_t bytes = (size_t)(l2 > 0 ? l2 : (128 << 20)) * 2;
        b->flush_n4 = bytes / sizeof(float4);
        WC_TRY(dalloc(&b->flush_buf, b->flush_n4));
        WC_TRY(dalloc(&b->flush_sink, 1));
        WC_CUDA_TRY(cudaMemsetAsync(b->flush_buf, 0, bytes, b->stream));
    }
    b->in.dt = dt;
    std::vector<cudaEvent_t> ev(2 * (size_t)nsteps, nullptr);
    for (auto& e : ev) WC_CUDA_TRY(cudaEventCreate(&e));
    wc_status st = WC_OK;
    for (uint32_t s = 0; s < nsteps && st == WC_OK; ++s) {
        if (flush_l2) launch_l2_flush(b->flush_buf, b->flush_n4, b->flush_sink, b->stream);
        cudaEventRecord(ev[2 * s], b->stream);
        st = launch(b, b->in);
        cudaEventRecord(ev[2 * s + 1], b->stream);
    }
    if (st == WC_OK) st = read_errors(b);
    for (uint32_t s = 0; s < nsteps && st == WC_OK; ++s) cudaEventElapsedTime(&step_ms[s], ev[2 * s], ev[2 * s + 1]);
    for (auto& e : ev)
        if (e) cudaEventDestroy(e);
    return st;
}

WC_API wc_status wc_batch_device_buffers(wc_batch* b, wc_device_buffers* out) {
    clear_error();
    WC_TRY(require(b, false));
    if (!out) return fail(WC_ERR_INVALID_ARG, "null output");
    std::memset(out, 0, sizeof *out);
    out->state_pos_density = b->d.pos_a;
    out->state_vel_pressure = b->d.vel_a;
    out->sorted_pos_density = b->d.pos_b;
    out->sorted_vel_pressure = b->d.vel_b;
    out->cell_keys = b->d.keys;
    out->permutation = b->d.perm;
    out->cell_start = b->d.start;
    out->stream = b->stream;
    out->num_particles = (uint32_t)b->n;
    out->num_cells = b->d.num_cells;
    return WC_OK;
}

WC_API wc_status wc_batch_get_tuning(const wc_batch* b, wc_tuning* out) {
    clear_error();
    WC_TRY(require(b, false));
    if (!out) return fail(WC_ERR_INVALID_ARG, "null output");
    *out = b->tuning;
    return WC_OK;
}

WC_API wc_status wc_batch_set_tuning(wc_batch* b, const wc_tuning* t) {
    clear_error();
    WC_TRY(require(b, false));
    if (!t || !(t->cell_factor >= 1.0f) || t->cell_factor > 4.0f)
        return fail(WC_ERR_INVALID_ARG, "cell_factor must be in [1, 4]");
    if (t->cell_factor != b->tuning.cell_factor) WC_TRY(apply_cell_factor(b, t->cell_factor));
    apply_geometry(b, *t);
    b->tuning.step_ms = t->step_ms;
    b->tuning.trials = t->trials;
    return WC_OK;
}

WC_API wc_status wc_batch_tune(wc_batch* b, float dt, wc_tuning* out) {
    clear_error();
    WC_NVTX("wc_batch_tune");
    WC_TRY(require(b, true));
    const TuneKey key{b->n, b->cells_cap};
    wc_tuning cached;
    if (cache_lookup(key, &cached)) {
        WC_TRY(wc_batch_set_tuning(b, &cached));
        if (out) *out = b->tuning;
        return WC_OK;
    }
    StepInputs in = b->in;
    in.dt = dt;
    WC_TRY(save_state(b));
    wc_tuning best = b->tuning;
    float best_ms = 1e30f;
    uint32_t trials = 0;
    auto trial = [&](const wc_tuning& t) -> wc_status {
        WC_TRY(wc_batch_set_tuning(b, &t));
        WC_TRY(restore_state(b));
        float ms = 0.f;
        WC_TRY(time_replays(b, in, 1, 3, &ms));
        ++trials;
        if (ms < best_ms) {
            best_ms = ms;
            best = b->tuning;
        }
        return WC_OK;
    };
    // Coordinate descent: cell size, then each kernel's resident blocks per SM.
    for (float f : {1.0f, 1.25f}) {
        wc_tuning t = best;
        t.cell_factor = f;
        WC_TRY(trial(t));
    }
    for (int blocks = b->max_density_blocks; blocks >= 1; --blocks) {
        wc_tuning t = best;
        t.density_blocks_per_sm = (uint32_t)blocks;
        WC_TRY(trial(t));
    }
    // threads per cell of both neighbour passes: a 32-lane team per cell or one lane per target, each
    // at its own largest residency
    for (uint32_t variant : {(uint32_t)WC_PASSES_LANE, (uint32_t)WC_PASSES_TEAM}) {
        wc_tuning t = best;
        t.pass_variant = variant;
        t.force_blocks_per_sm = 64;  // clamped to the variant's occupancy
        WC_TRY(trial(t));
    }
    {
        wc_tuning probe = best;
        WC_TRY(wc_batch_set_tuning(b, &probe));  // max_force_blocks of the chosen variant
    }
    for (int blocks = b->max_force_blocks; blocks >= 1; --blocks) {
        wc_tuning t = best;
        t.force_blocks_per_sm = (uint32_t)blocks;
        WC_TRY(trial(t));
    }
    for (uint32_t blocks : {4u, 8u, 16u}) {
        wc_tuning t = best;
        t.stream_blocks_per_sm = blocks;
        WC_TRY(trial(t));
    }
    best.step_ms = best_ms;
    best.trials = trials;
    WC_TRY(wc_batch_set_tuning(b, &best));
    WC_TRY(restore_state(b));
    WC_CUDA_TRY(cudaStreamSynchronize(b->stream));
    cache_store(key, best);
    if (out) *out = best;
    return WC_OK;
}

}  // extern "C"
