// wc_fluid.cu — the wc_fluid handle: the GB300 replacement of core::Fluid + core::Sort
// (src/core/Fluid.{h,cpp}, src/core/Sort.{h,cpp}). It owns every device buffer, enqueues the
// six kernels of a step on its own stream, and replays them as one CUDA graph per update.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "wc_internal.h"
#include "wc_util.h"

using namespace wc;

namespace {

constexpr uint32_t NUM_STEP_KERNELS = 6;
const char* const STEP_KERNEL_NAMES[NUM_STEP_KERNELS] = {"bin_count", "scan_cells",     "scatter_cells",
                                                         "rank_gather", "density", "force_integrate"};

bool same_inputs(const StepInputs& a, const StepInputs& b) { return std::memcmp(&a, &b, sizeof a) == 0; }

}  // namespace

struct wc_fluid {
    wc_params params{};
    SceneConsts sc{};
    StepInputs in{};
    DevBuffers d{};
    LaunchDims ld{};
    int device = 0;
    cudaStream_t stream = nullptr;
    bool setup_done = false;
    uint64_t steps = 0;
    // step graph
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphNode_t force_node = nullptr;
    cudaKernelNodeParams force_params{};
    ForceKernelArgs fargs{};
    StepInputs graph_in{};
    // host-copy staging (AoS, 32 bytes per particle) and error word
    float4* staging = nullptr;
    uint32_t* h_err = nullptr;
    HostReadback readback{};  // wc_fluid_update_host
    // L2 flush for timing
    float4* flush_buf = nullptr;
    size_t flush_n4 = 0;
    float* flush_sink = nullptr;
};

namespace {

template <class T>
wc_status dalloc(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) return WC_OK;
    WC_TRY(::wc::device_alloc(reinterpret_cast<void**>(p), count * sizeof(T)));
    return WC_OK;
}

void free_all(wc_fluid* f) {
    DevBuffers& d = f->d;
    void* ptrs[] = {d.pos_a,     d.vel_a,        d.pos_b,     d.vel_b,    d.ids_a,           d.ids_b,
                    d.keys,      d.ranks,        d.unordered, d.perm,     d.counts,          d.start,
                    d.cell_list, d.num_nonempty, d.scan_desc, d.ncount,   d.scan_tile_counter, d.err,
                    d.hits,      f->staging,     f->flush_buf, f->flush_sink, d.accel,  d.xyz};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (f->h_err) cudaFreeHost(f->h_err);
    if (f->exec) cudaGraphExecDestroy(f->exec);
    if (f->graph) cudaGraphDestroy(f->graph);
    f->readback.release();
    if (f->stream) cudaStreamDestroy(f->stream);
}

wc_status allocate(wc_fluid* f) {
    DevBuffers& d = f->d;
    const uint32_t n = f->params.num_particles;
    const uint32_t R = f->params.grid_res;
    d.n = n;
    d.num_cells = R * R * R;
    d.num_tiles = (d.num_cells + SCAN_TILE - 1) / SCAN_TILE;
    WC_TRY(dalloc(&d.pos_a, n));
    WC_TRY(dalloc(&d.vel_a, n));
    WC_TRY(dalloc(&d.pos_b, n));
    WC_TRY(dalloc(&d.vel_b, n));
    if (f->params.flags & WC_FLAG_TRACK_IDS) {
        WC_TRY(dalloc(&d.ids_a, n));
        WC_TRY(dalloc(&d.ids_b, n));
    }
    WC_TRY(dalloc(&d.keys, n));
    WC_TRY(dalloc(&d.ranks, n));
    WC_TRY(dalloc(&d.unordered, n));
    WC_TRY(dalloc(&d.perm, n));
    if (f->params.flags & WC_FLAG_NEIGHBOR_COUNTS) WC_TRY(dalloc(&d.ncount, n));
    WC_TRY(dalloc(&d.hits, (size_t)n * MASK_WORDS));
    d.xyz_stride = xyz_stride_for(n);
    WC_TRY(dalloc(&d.xyz, 3 * (size_t)d.xyz_stride));
    WC_TRY(dalloc(&d.counts, d.num_cells));
    WC_TRY(dalloc(&d.start, (size_t)d.num_cells + 1));
    WC_TRY(dalloc(&d.cell_list, d.num_cells));
    WC_TRY(dalloc(&d.num_nonempty, 3));
    WC_TRY(dalloc(&d.scan_desc, d.num_tiles));
    WC_TRY(dalloc(&d.scan_tile_counter, 1));
    WC_TRY(dalloc(&d.err, 1));
    WC_CUDA_TRY(cudaMallocHost(reinterpret_cast<void**>(&f->h_err), sizeof(uint32_t)));
    WC_CUDA_TRY(cudaMemsetAsync(d.counts, 0, sizeof(uint32_t) * d.num_cells, f->stream));
    WC_CUDA_TRY(cudaMemsetAsync(d.start, 0, sizeof(uint32_t) * ((size_t)d.num_cells + 1), f->stream));
    WC_CUDA_TRY(cudaMemsetAsync(d.num_nonempty, 0, 3 * sizeof(uint32_t), f->stream));
    WC_CUDA_TRY(cudaMemsetAsync(d.err, 0, sizeof(uint32_t), f->stream));
    WC_CUDA_TRY(cudaMemsetAsync(d.xyz, 0, sizeof(float) * 3 * (size_t)d.xyz_stride, f->stream));
    if (n) {
        WC_CUDA_TRY(cudaMemsetAsync(d.pos_a, 0, sizeof(float4) * n, f->stream));
        WC_CUDA_TRY(cudaMemsetAsync(d.vel_a, 0, sizeof(float4) * n, f->stream));
        WC_CUDA_TRY(cudaMemsetAsync(d.pos_b, 0, sizeof(float4) * n, f->stream));
        WC_CUDA_TRY(cudaMemsetAsync(d.vel_b, 0, sizeof(float4) * n, f->stream));
        WC_CUDA_TRY(cudaMemsetAsync(d.perm, 0, sizeof(uint32_t) * n, f->stream));
        WC_CUDA_TRY(cudaMemsetAsync(d.keys, 0, sizeof(uint32_t) * n, f->stream));
        if (d.ncount) WC_CUDA_TRY(cudaMemsetAsync(d.ncount, 0, sizeof(uint32_t) * n, f->stream));
        WC_CUDA_TRY(cudaMemsetAsync(d.hits, 0, sizeof(uint32_t) * MASK_WORDS * (size_t)n, f->stream));
    }
    WC_CUDA_TRY(cudaStreamSynchronize(f->stream));
    return WC_OK;
}

wc_status ensure_staging(wc_fluid* f) {
    if (!f->staging && f->d.n) WC_TRY(dalloc(&f->staging, 2 * (size_t)f->d.n));
    return WC_OK;
}

__global__ void iota_kernel(uint32_t* __restrict__ out, uint32_t n);
wc_status check_launch();

// Host AoS -> the state (or sorted) buffer, on the fluid's stream, without waiting: the caller
// waits before the host buffer may change.
wc_status enqueue_upload(wc_fluid* f, bool state, const wc_particle* in, uint32_t n) {
    WC_TRY(ensure_staging(f));
    WC_CUDA_TRY(cudaMemcpyAsync(f->staging, in, sizeof(wc_particle) * (size_t)n, cudaMemcpyHostToDevice, f->stream));
    launch_aos_to_soa(f->staging, state ? f->d.pos_a : f->d.pos_b, state ? f->d.vel_a : f->d.vel_b, n, f->stream);
    WC_TRY(check_launch());
    if (state && f->d.ids_a) {
        // tracked ids restart at the uploaded order
        iota_kernel<<<(n + 1023) / 1024, 256, 0, f->stream>>>(f->d.ids_a, n);
        WC_TRY(check_launch());
    }
    return WC_OK;
}

void enqueue_sort(wc_fluid* f) {
    launch_bin_count(f->d, f->sc, f->ld, f->stream);
    launch_scan_cells(f->d, f->stream);
    launch_scatter(f->d, f->ld, f->stream);
    launch_rank_gather(f->d, f->ld, f->stream);
}

void enqueue_step(wc_fluid* f, const StepInputs& in) {
    enqueue_sort(f);
    launch_density(f->d, f->sc, f->ld, f->stream);
    launch_force(f->d, f->sc, in, f->ld, f->stream);
}

wc_status check_launch() {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(WC_ERR_CUDA, "kernel launch failed: %s", cudaGetErrorString(e));
    return WC_OK;
}

wc_status capture_graph(wc_fluid* f, const StepInputs& in) {
    WC_CUDA_TRY(cudaStreamBeginCapture(f->stream, cudaStreamCaptureModeThreadLocal));
    enqueue_step(f, in);
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(f->stream, &g);
    if (ce != cudaSuccess) return fail(WC_ERR_CUDA, "step graph capture failed: %s", cudaGetErrorString(ce));
    f->graph = g;
    WC_CUDA_TRY(cudaGraphInstantiate(&f->exec, g, 0));
    size_t count = 0;
    WC_CUDA_TRY(cudaGraphGetNodes(g, nullptr, &count));
    std::vector<cudaGraphNode_t> nodes(count);
    WC_CUDA_TRY(cudaGraphGetNodes(g, nodes.data(), &count));
    const void* force_fn = force_kernel_symbol(f->ld.pass_variant);
    for (cudaGraphNode_t nd : nodes) {
        cudaGraphNodeType ty;
        WC_CUDA_TRY(cudaGraphNodeGetType(nd, &ty));
        if (ty != cudaGraphNodeTypeKernel) continue;
        cudaKernelNodeParams kp;
        WC_CUDA_TRY(cudaGraphKernelNodeGetParams(nd, &kp));
        if (kp.func == force_fn) {
            f->force_node = nd;
            f->force_params = kp;
        }
    }
    if (!f->force_node) return fail(WC_ERR_CUDA, "step graph has no force node");
    ForceKernelArgs& a = f->fargs;
    a.sc = f->sc;
    a.bt = BatchTables{};
    a.in = in;
    a.n = f->d.n;
    a.num_cells = f->d.num_cells;
    a.pos_b = f->d.pos_b;
    a.vel_b = f->d.vel_b;
    a.ids_b = f->d.ids_b;
    a.pos_a = f->d.pos_a;
    a.vel_a = f->d.vel_a;
    a.ids_a = f->d.ids_a;
    a.start = f->d.start;
    a.cell_list = f->d.cell_list;
    a.num_nonempty = f->d.num_nonempty;
    a.hits = f->d.hits;
    a.accel = f->d.accel;
    a.err = f->d.err;
    a.bind();
    f->graph_in = in;
    return WC_OK;
}

wc_status launch_step(wc_fluid* f, const StepInputs& in) {
    if (!f->exec) {
        WC_TRY(capture_graph(f, in));
    } else if (!same_inputs(in, f->graph_in)) {
        f->fargs.in = in;
        cudaKernelNodeParams kp = f->force_params;
        kp.kernelParams = f->fargs.ptrs;
        kp.extra = nullptr;
        WC_CUDA_TRY(cudaGraphExecKernelNodeSetParams(f->exec, f->force_node, &kp));
        f->graph_in = in;
    }
    WC_CUDA_TRY(cudaGraphLaunch(f->exec, f->stream));
    ++f->steps;
    return WC_OK;
}

wc_status read_device_errors(wc_fluid* f) {
    // the copy follows everything already on the stream: one wait covers both
    WC_CUDA_TRY(cudaMemcpyAsync(f->h_err, f->d.err, sizeof(uint32_t), cudaMemcpyDeviceToHost, f->stream));
    WC_CUDA_TRY(cudaStreamSynchronize(f->stream));
    const uint32_t e = *f->h_err;
    if (e) {
        WC_CUDA_TRY(cudaMemsetAsync(f->d.err, 0, sizeof(uint32_t), f->stream));
        WC_CUDA_TRY(cudaStreamSynchronize(f->stream));
        if (e & DEVERR_SCAN_TIMEOUT)
            return fail(WC_ERR_TIMEOUT, "cell scan look-back exceeded its wait limit; tables of that step are invalid");
        if (e & DEVERR_CELL_OVERFLOW)
            return fail(WC_ERR_NUMERIC, "a cell held more than %u particles (a collapsed or non-finite state); its "
                                        "particles were not evaluated", MAX_CELL_PARTICLES);
        return fail(WC_ERR_NUMERIC, "a particle position was NaN or infinite when it was binned");
    }
    return WC_OK;
}

wc_status require(const wc_fluid* f, bool need_setup) {
    if (!f) return fail(WC_ERR_INVALID_ARG, "null fluid handle");
    if (need_setup && !f->setup_done) return fail(WC_ERR_STATE, "wc_fluid_setup has not been called");
    return WC_OK;
}

__global__ void iota_kernel(uint32_t* __restrict__ out, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = i;
}

}  // namespace

namespace wc {

wc_status HostReadback::arm(cudaStream_t s, uint32_t n, float4* staging, StepInputs& step) {
    if (!copy_stream) WC_CUDA_TRY(cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking));
    if (!part_done) {
        WC_TRY(dalloc(&part_done, READBACK_PARTS));
        WC_CUDA_TRY(cudaMemsetAsync(part_done, 0, sizeof(uint32_t) * READBACK_PARTS, s));
    }
    if (!part_flag) {
        WC_CUDA_TRY(cudaHostAlloc(reinterpret_cast<void**>(&part_flag), sizeof(uint32_t) * READBACK_PARTS,
                                  cudaHostAllocMapped));
        std::memset(part_flag, 0, sizeof(uint32_t) * READBACK_PARTS);
        WC_CUDA_TRY(cudaHostGetDevicePointer(reinterpret_cast<void**>(&part_flag_dev), part_flag, 0));
    }
    if (++seq == 0) ++seq;  // the flags start at 0: no launch publishes 0
    const uint32_t chunks = (n + 31u) >> 5;
    part_chunks = (chunks + READBACK_PARTS - 1) / READBACK_PARTS;
    parts = (chunks + part_chunks - 1) / part_chunks;
    step.aos_out = staging;  // the pass writes the host records itself: no conversion kernel
    step.part_done = part_done;
    step.part_flag = part_flag_dev;
    step.part_chunks = part_chunks;
    step.seq = seq;
    return WC_OK;
}

wc_status HostReadback::drain(cudaStream_t s, uint32_t n, const float4* staging, wc_particle* out) {
    const volatile uint32_t* flag = part_flag;
    for (uint32_t r = 0; r < parts; ++r) {
        // part r is published once its last chunk is stored; a stream that has ended (or failed)
        // without the flag ends the wait too, and the copy then reads what the stream left
        for (uint32_t spin = 1; flag[r] != seq; ++spin)
            if ((spin & 1023u) == 0u && cudaStreamQuery(s) != cudaErrorNotReady) break;
        const uint32_t s0 = r * part_chunks * 32u, s1 = std::min((r + 1) * part_chunks * 32u, n);
        WC_CUDA_TRY(cudaMemcpyAsync(out + s0, staging + 2 * (size_t)s0, sizeof(wc_particle) * (size_t)(s1 - s0),
                                    cudaMemcpyDeviceToHost, copy_stream));
    }
    WC_CUDA_TRY(cudaStreamSynchronize(copy_stream));
    return WC_OK;
}

void HostReadback::release() {
    if (part_done) cudaFree(part_done);
    if (part_flag) cudaFreeHost(part_flag);
    if (copy_stream) cudaStreamDestroy(copy_stream);
    *this = HostReadback{};
}

FluidInternals fluid_internals(wc_fluid* f) {
    return FluidInternals{&f->d, &f->sc, &f->in, &f->params, f->stream};
}

void fluid_enqueue_sort(wc_fluid* f) { enqueue_sort(f); }

StepTarget fluid_target(wc_fluid* f) {
    StepTarget t{};
    t.d = &f->d;
    t.sc = f->sc;
    t.in = &f->in;
    t.ld = f->ld;
    t.stream = f->stream;
    t.fluid = f;
    return t;
}

wc_status fluid_check(wc_fluid* f) {
    WC_TRY(check_launch());
    return read_device_errors(f);
}

wc_status fluid_graph_step(wc_fluid* f, float dt) {
    // the caller counts its own steps (a judged rollout step runs this and a candidate)
    const uint64_t steps = f->steps;
    f->in.dt = dt;
    const wc_status rc = launch_step(f, f->in);
    f->steps = steps;
    return rc;
}

void fluid_count_step(wc_fluid* f) { ++f->steps; }
void fluid_set_step_count(wc_fluid* f, uint64_t steps) { f->steps = steps; }

}  // namespace wc

extern "C" {

WC_API wc_status wc_fluid_create(const wc_params* p, wc_fluid** out) {
    clear_error();
    if (!p || !out) return fail(WC_ERR_INVALID_ARG, "wc_fluid_create: null argument");
    *out = nullptr;
    wc_params prm = *p;
    WC_TRY(wc_params_finalize(&prm));
    int ndev = 0;
    const cudaError_t de = cudaGetDeviceCount(&ndev);
    if (de != cudaSuccess || ndev == 0)
        return fail(WC_ERR_CUDA, "no CUDA device: %s", de != cudaSuccess ? cudaGetErrorString(de) : "count is 0");
    wc_fluid* f = new (std::nothrow) wc_fluid();
    if (!f) return fail(WC_ERR_OOM, "host allocation failed");
    f->params = prm;
    cudaGetDevice(&f->device);
    wc_status s = WC_OK;
    if (cudaStreamCreateWithFlags(&f->stream, cudaStreamNonBlocking) != cudaSuccess) {
        s = fail(WC_ERR_CUDA, "stream creation failed");
    } else {
        s = allocate(f);
    }
    if (s != WC_OK) {
        free_all(f);
        delete f;
        return s;
    }
    f->ld = compute_launch_dims(f->device, (f->params.flags & WC_FLAG_CELL_TEAMS) ? PASSES_TEAM : PASSES_LANE);
    f->sc = make_scene_consts(prm);
    f->in = make_step_inputs(prm, 0.0f);
    *out = f;
    return WC_OK;
}

WC_API void wc_fluid_destroy(wc_fluid* f) {
    if (!f) return;
    if (f->stream) cudaStreamSynchronize(f->stream);
    free_all(f);
    delete f;
}

WC_API wc_status wc_fluid_setup(wc_fluid* f, const wc_particle* initial, uint32_t n) {
    clear_error();
    WC_NVTX("wc_fluid_setup");
    WC_TRY(require(f, false));
    if (n != f->d.n) return fail(WC_ERR_INVALID_ARG, "setup with %u particles, handle holds %u", n, f->d.n);
    if (n && !initial) return fail(WC_ERR_INVALID_ARG, "null initial particles");
    if (n) WC_TRY(wc_fluid_set_particles(f, WC_BUFFER_STATE, initial, n));
    f->setup_done = true;
    f->steps = 0;
    return WC_OK;
}

WC_API wc_status wc_fluid_update(wc_fluid* f, double time) {
    clear_error();
    WC_NVTX("wc_fluid_update");
    WC_TRY(require(f, true));
    const float dt = (float)time * f->params.time_scale;  // Fluid.cpp:308
    f->in.dt = dt;
    return launch_step(f, f->in);
}

WC_API wc_status wc_fluid_step(wc_fluid* f, float dt, uint32_t nsteps) {
    clear_error();
    WC_NVTX("wc_fluid_step");
    WC_TRY(require(f, true));
    f->in.dt = dt;
    for (uint32_t s = 0; s < nsteps; ++s) WC_TRY(launch_step(f, f->in));
    return WC_OK;
}

WC_API wc_status wc_fluid_sort(wc_fluid* f) {
    clear_error();
    WC_NVTX("wc_fluid_sort");
    WC_TRY(require(f, true));
    enqueue_sort(f);
    return check_launch();
}

WC_API wc_status wc_fluid_density(wc_fluid* f) {
    clear_error();
    WC_NVTX("wc_fluid_density");
    WC_TRY(require(f, true));
    launch_density(f->d, f->sc, f->ld, f->stream);
    return check_launch();
}

WC_API wc_status wc_fluid_integrate(wc_fluid* f, float dt) {
    clear_error();
    WC_NVTX("wc_fluid_integrate");
    WC_TRY(require(f, true));
    StepInputs in = f->in;
    in.dt = dt;
    launch_force(f->d, f->sc, in, f->ld, f->stream);
    WC_TRY(check_launch());
    ++f->steps;
    return WC_OK;
}

WC_API wc_status wc_fluid_set_mouse_ray(wc_fluid* f, const float origin[3], const float dir[3]) {
    clear_error();
    WC_TRY(require(f, false));
    if (!origin || !dir) return fail(WC_ERR_INVALID_ARG, "null mouse ray");
    for (int a = 0; a < 3; ++a) {
        f->in.mouse_o[a] = f->params.mouse_origin[a] = origin[a];
        f->in.mouse_d[a] = f->params.mouse_dir[a] = dir[a];
    }
    return WC_OK;
}

WC_API wc_status wc_fluid_set_gravity(wc_fluid* f, const float gravity[3]) {
    clear_error();
    WC_TRY(require(f, false));
    if (!gravity) return fail(WC_ERR_INVALID_ARG, "null gravity");
    for (int a = 0; a < 3; ++a) f->in.g[a] = f->params.gravity[a] = gravity[a];
    return WC_OK;
}

WC_API wc_status wc_fluid_get_particles(wc_fluid* f, int buffer, wc_particle* out, uint32_t n) {
    clear_error();
    WC_NVTX("wc_fluid_get_particles");
    WC_TRY(require(f, false));
    if (buffer != WC_BUFFER_STATE && buffer != WC_BUFFER_SORTED)
        return fail(WC_ERR_INVALID_ARG, "unknown buffer %d", buffer);
    if (n != f->d.n) return fail(WC_ERR_INVALID_ARG, "copy of %u particles, handle holds %u", n, f->d.n);
    if (!n) return read_device_errors(f);
    if (!out) return fail(WC_ERR_INVALID_ARG, "null output");
    const bool st = buffer == WC_BUFFER_STATE;
    WC_TRY(ensure_staging(f));
    launch_soa_to_aos(st ? f->d.pos_a : f->d.pos_b, st ? f->d.vel_a : f->d.vel_b, f->staging, n, f->stream);
    WC_TRY(check_launch());
    WC_CUDA_TRY(cudaMemcpyAsync(out, f->staging, sizeof(wc_particle) * (size_t)n, cudaMemcpyDeviceToHost, f->stream));
    return read_device_errors(f);
}

WC_API wc_status wc_fluid_set_particles(wc_fluid* f, int buffer, const wc_particle* in, uint32_t n) {
    clear_error();
    WC_NVTX("wc_fluid_set_particles");
    WC_TRY(require(f, false));
    if (buffer != WC_BUFFER_STATE && buffer != WC_BUFFER_SORTED)
        return fail(WC_ERR_INVALID_ARG, "unknown buffer %d", buffer);
    if (n != f->d.n) return fail(WC_ERR_INVALID_ARG, "copy of %u particles, handle holds %u", n, f->d.n);
    if (!n) return WC_OK;
    if (!in) return fail(WC_ERR_INVALID_ARG, "null input");
    WC_TRY(enqueue_upload(f, buffer == WC_BUFFER_STATE, in, n));
    // The host buffer may be reused as soon as this returns.
    WC_CUDA_TRY(cudaStreamSynchronize(f->stream));
    return WC_OK;
}

WC_API wc_status wc_fluid_update_host(wc_fluid* f, double time, const wc_particle* in, wc_particle* out, uint32_t n) {
    clear_error();
    WC_NVTX("wc_fluid_update_host");
    WC_TRY(require(f, true));
    if (n != f->d.n) return fail(WC_ERR_INVALID_ARG, "copy of %u particles, handle holds %u", n, f->d.n);
    if (!n || !out || f->ld.pass_variant != PASSES_LANE) {
        // nothing to overlap: the three calls in turn
        if (n && in) WC_TRY(wc_fluid_set_particles(f, WC_BUFFER_STATE, in, n));
        WC_TRY(wc_fluid_update(f, time));
        return out ? wc_fluid_get_particles(f, WC_BUFFER_STATE, out, n) : WC_OK;
    }
    f->in.dt = (float)time * f->params.time_scale;  // Fluid.cpp:308
    if (in) WC_TRY(enqueue_upload(f, true, in, n));  // the final wait covers the copy from in
    WC_TRY(ensure_staging(f));
    StepInputs step = f->in;
    WC_TRY(f->readback.arm(f->stream, n, f->staging, step));
    // the step of the graph, launched directly with the readback fields
    enqueue_sort(f);
    launch_density(f->d, f->sc, f->ld, f->stream);
    launch_force(f->d, f->sc, step, f->ld, f->stream);
    WC_TRY(check_launch());
    WC_TRY(f->readback.drain(f->stream, n, f->staging, out));
    ++f->steps;
    return read_device_errors(f);
}

WC_API wc_status wc_fluid_get_uints(wc_fluid* f, int which, uint32_t* out, size_t n) {
    clear_error();
    WC_TRY(require(f, false));
    if (!out && n) return fail(WC_ERR_INVALID_ARG, "null output");
    const DevBuffers& d = f->d;
    const uint32_t* src = nullptr;
    size_t len = d.n;
    switch (which) {
        case WC_UINTS_CELL_KEYS: src = d.keys; break;
        case WC_UINTS_PERMUTATION: src = d.perm; break;
        case WC_UINTS_NEIGHBOR_COUNTS:
            if (!d.ncount) return fail(WC_ERR_STATE, "neighbour counts need WC_FLAG_NEIGHBOR_COUNTS");
            src = d.ncount;
            break;
        case WC_UINTS_PARTICLE_IDS:
            if (!d.ids_a) return fail(WC_ERR_STATE, "particle ids need WC_FLAG_TRACK_IDS");
            src = d.ids_a;
            break;
        case WC_UINTS_CELL_COUNTS:
        case WC_UINTS_CELL_OFFSETS: {
            len = d.num_cells;
            if (n != len) return fail(WC_ERR_INVALID_ARG, "cell table has %zu entries, asked for %zu", len, n);
            std::vector<uint32_t> st((size_t)d.num_cells + 1);
            WC_CUDA_TRY(cudaMemcpyAsync(st.data(), d.start, sizeof(uint32_t) * st.size(), cudaMemcpyDeviceToHost,
                                        f->stream));
            WC_TRY(read_device_errors(f));
            for (size_t c = 0; c < len; ++c) out[c] = which == WC_UINTS_CELL_OFFSETS ? st[c] : st[c + 1] - st[c];
            return WC_OK;
        }
        default: return fail(WC_ERR_INVALID_ARG, "unknown uint buffer %d", which);
    }
    if (n != len) return fail(WC_ERR_INVALID_ARG, "buffer has %zu entries, asked for %zu", len, n);
    if (len) WC_CUDA_TRY(cudaMemcpyAsync(out, src, sizeof(uint32_t) * len, cudaMemcpyDeviceToHost, f->stream));
    return read_device_errors(f);
}

WC_API wc_status wc_fluid_get_params(const wc_fluid* f, wc_params* out) {
    clear_error();
    if (!f || !out) return fail(WC_ERR_INVALID_ARG, "null argument");
    *out = f->params;
    return WC_OK;
}

WC_API wc_status wc_fluid_get_device_buffers(wc_fluid* f, wc_device_buffers* out) {
    clear_error();
    WC_TRY(require(f, false));
    if (!out) return fail(WC_ERR_INVALID_ARG, "null output");
    std::memset(out, 0, sizeof *out);
    out->state_pos_density = f->d.pos_a;
    out->state_vel_pressure = f->d.vel_a;
    out->sorted_pos_density = f->d.pos_b;
    out->sorted_vel_pressure = f->d.vel_b;
    out->cell_keys = f->d.keys;
    out->permutation = f->d.perm;
    out->cell_start = f->d.start;
    out->neighbor_counts = f->d.ncount;
    out->particle_ids = f->d.ids_a;
    out->stream = f->stream;
    out->num_particles = f->d.n;
    out->num_cells = f->d.num_cells;
    return WC_OK;
}

WC_API wc_status wc_fluid_synchronize(wc_fluid* f) {
    clear_error();
    WC_TRY(require(f, false));
    WC_TRY(check_launch());
    return read_device_errors(f);
}

WC_API uint64_t wc_fluid_step_count(const wc_fluid* f) { return f ? f->steps : 0; }

WC_API wc_status wc_fluid_set_recording(wc_fluid* f, int on) {
    clear_error();
    WC_TRY(require(f, false));
    if (on && !f->d.accel) {
        WC_TRY(dalloc(&f->d.accel, f->d.n));
        if (f->d.n) WC_CUDA_TRY(cudaMemsetAsync(f->d.accel, 0, sizeof(float4) * f->d.n, f->stream));
    } else if (!on && f->d.accel) {
        WC_CUDA_TRY(cudaStreamSynchronize(f->stream));
        cudaFree(f->d.accel);
        f->d.accel = nullptr;
    }
    if (f->exec) cudaGraphExecDestroy(f->exec);
    if (f->graph) cudaGraphDestroy(f->graph);
    f->exec = nullptr;
    f->graph = nullptr;
    f->force_node = nullptr;
    return WC_OK;
}

WC_API wc_status wc_fluid_get_accelerations(wc_fluid* f, float* out, uint32_t n) {
    clear_error();
    WC_TRY(require(f, false));
    if (!f->d.accel) return fail(WC_ERR_STATE, "recording is off (wc_fluid_set_recording)");
    if (n != f->d.n || (!out && n)) return fail(WC_ERR_INVALID_ARG, "bad acceleration buffer");
    if (n) WC_CUDA_TRY(cudaMemcpyAsync(out, f->d.accel, sizeof(float4) * n, cudaMemcpyDeviceToHost, f->stream));
    return read_device_errors(f);
}

WC_API uint32_t wc_step_kernel_count(void) { return NUM_STEP_KERNELS; }

WC_API const char* wc_step_kernel_name(uint32_t index) {
    return index < NUM_STEP_KERNELS ? STEP_KERNEL_NAMES[index] : "";
}

WC_API wc_status wc_fluid_time_steps(wc_fluid* f, float dt, uint32_t nsteps, int flush_l2, float* step_ms,
                                     float* kernel_ms) {
    clear_error();
    WC_NVTX("wc_fluid_time_steps");
    WC_TRY(require(f, true));
    if (!step_ms && !kernel_ms && nsteps) return fail(WC_ERR_INVALID_ARG, "null step_ms and kernel_ms");
    if (flush_l2 && !f->flush_buf) {
        int l2 = 0;
        cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, f->device);
        const size_t bytes = (size_t)(l2 > 0 ? l2 : (128 << 20)) * 2;
        f->flush_n4 = bytes / sizeof(float4);
        WC_TRY(dalloc(&f->flush_buf, f->flush_n4));
        WC_TRY(dalloc(&f->flush_sink, 1));
        WC_CUDA_TRY(cudaMemsetAsync(f->flush_buf, 0, bytes, f->stream));
    }
    f->in.dt = dt;
    std::vector<cudaEvent_t> ev(2 * (size_t)nsteps + 7, nullptr);
    for (auto& e : ev) WC_CUDA_TRY(cudaEventCreate(&e));
    wc_status st = WC_OK;
    if (step_ms) {
        for (uint32_t s = 0; s < nsteps && st == WC_OK; ++s) {
            if (flush_l2) launch_l2_flush(f->flush_buf, f->flush_n4, f->flush_sink, f->stream);
            cudaEventRecord(ev[2 * s], f->stream);
            st = launch_step(f, f->in);
            cudaEventRecord(ev[2 * s + 1], f->stream);
        }
        if (st == WC_OK) st = read_device_errors(f);
        for (uint32_t s = 0; s < nsteps && st == WC_OK; ++s) {
            float ms = 0.f;
            cudaEventElapsedTime(&ms, ev[2 * s], ev[2 * s + 1]);
            step_ms[s] = ms;
        }
    }
    if (st == WC_OK && kernel_ms) {
        cudaEvent_t* ke = ev.data() + 2 * (size_t)nsteps;  // 7 events: around and between kernels
        for (uint32_t s = 0; s < nsteps && st == WC_OK; ++s) {
            if (flush_l2) launch_l2_flush(f->flush_buf, f->flush_n4, f->flush_sink, f->stream);
            cudaEventRecord(ke[0], f->stream);
            launch_bin_count(f->d, f->sc, f->ld, f->stream);
            cudaEventRecord(ke[1], f->stream);
            launch_scan_cells(f->d, f->stream);
            cudaEventRecord(ke[2], f->stream);
            launch_scatter(f->d, f->ld, f->stream);
            cudaEventRecord(ke[3], f->stream);
            launch_rank_gather(f->d, f->ld, f->stream);
            cudaEventRecord(ke[4], f->stream);
            launch_density(f->d, f->sc, f->ld, f->stream);
            cudaEventRecord(ke[5], f->stream);
            launch_force(f->d, f->sc, f->in, f->ld, f->stream);
            cudaEventRecord(ke[6], f->stream);
            ++f->steps;
            st = check_launch();
            if (st == WC_OK) st = read_device_errors(f);
            for (uint32_t k = 0; k < NUM_STEP_KERNELS && st == WC_OK; ++k)
                cudaEventElapsedTime(&kernel_ms[(size_t)s * NUM_STEP_KERNELS + k], ke[k], ke[k + 1]);
        }
    }
    for (auto& e : ev)
        if (e) cudaEventDestroy(e);
    return st;
}

WC_API wc_status wc_set_device(int device) {
    clear_error();
    WC_CUDA_TRY(cudaSetDevice(device));
    return WC_OK;
}

WC_API int wc_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
    return n;
}

WC_API wc_status wc_alloc_host(size_t bytes, void** out) {
    clear_error();
    if (!out) return fail(WC_ERR_INVALID_ARG, "null output");
    *out = nullptr;
    if (!bytes) return WC_OK;
    WC_CUDA_TRY(cudaMallocHost(out, bytes));
    return WC_OK;
}

WC_API void wc_free_host(void* p) {
    if (p) cudaFreeHost(p);
}

}  // extern "C"
