// wc_snapshot.cu — binary snapshots of a fluid's state for resume, rollouts and training data.
// No counterpart in the reference (its reset() is a no-op, src/core/Fluid.h:57).
//
// File layout (little-endian, as the structs lie in memory):
//   wc_snapshot_header                      (magic, version, sizes, step, seed, parameters)
//   float4 pos_density[n]                   state buffer: x, y, z, density
//   float4 vel_pressure[n]                  state buffer: vx, vy, vz, pressure
//   uint32 ids[n]                           only when header.has_ids
//   uint64 checksum                         FNV-1a 64 of every byte before it
// The state buffer is stored in the order of the last sort, exactly as the solver holds it, so
// a fluid loaded from a snapshot continues bit for bit where the saved one stopped.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <vector>

#include "wc_internal.h"
#include "wc_util.h"

using namespace wc;

namespace {

constexpr char MAGIC[8] = {'W', 'C', 'S', 'N', 'A', 'P', '\0', '\1'};
constexpr uint32_t VERSION = 1;

uint64_t fnv1a(uint64_t h, const void* data, size_t n) {
    const unsigned char* p = static_cast<const unsigned char*>(data);
    for (size_t i = 0; i < n; ++i) {
        h ^= p[i];
        h *= 1099511628211ull;
    }
    return h;
}
constexpr uint64_t FNV_OFFSET = 14695981039346656037ull;

struct File {
    FILE* f = nullptr;
    ~File() {
        if (f) std::fclose(f);
    }
};

// The parameters a loaded snapshot must share with the handle: everything but the gravity and
// mouse ray, which the load applies (they change between steps without a new handle).
bool same_fixed_params(wc_params a, wc_params b) {
    std::memset(a.gravity, 0, sizeof a.gravity);
    std::memset(b.gravity, 0, sizeof b.gravity);
    std::memset(a.mouse_origin, 0, sizeof a.mouse_origin);
    std::memset(b.mouse_origin, 0, sizeof b.mouse_origin);
    std::memset(a.mouse_dir, 0, sizeof a.mouse_dir);
    std::memset(b.mouse_dir, 0, sizeof b.mouse_dir);
    return std::memcmp(&a, &b, sizeof a) == 0;
}

// Reads and verifies a whole snapshot: header, body and checksum.
wc_status read_file(const char* path, wc_snapshot_header* hdr, std::vector<float4>* pos, std::vector<float4>* vel,
                    std::vector<uint32_t>* ids) {
    if (!path || !hdr) return fail(WC_ERR_INVALID_ARG, "null argument");
    File fh;
    fh.f = std::fopen(path, "rb");
    if (!fh.f) return fail(WC_ERR_INVALID_ARG, "cannot open snapshot '%s'", path);
    if (std::fread(hdr, sizeof *hdr, 1, fh.f) != 1) return fail(WC_ERR_INVALID_ARG, "snapshot '%s' is truncated", path);
    if (std::memcmp(hdr->magic, MAGIC, sizeof MAGIC) != 0) return fail(WC_ERR_INVALID_ARG, "'%s' is not a snapshot", path);
    if (hdr->version != VERSION || hdr->header_bytes != sizeof(wc_snapshot_header))
        return fail(WC_ERR_INVALID_ARG, "snapshot '%s' has version %u / header %u bytes (want %u / %zu)", path,
                    hdr->version, hdr->header_bytes, VERSION, sizeof(wc_snapshot_header));
    if (hdr->num_particles != hdr->params.num_particles || hdr->num_particles > 0xffffffffull || hdr->has_ids > 1)
        return fail(WC_ERR_INVALID_ARG, "snapshot '%s' has an inconsistent header", path);
    const size_t n = (size_t)hdr->num_particles;
    std::vector<float4> p(n), v(n);
    std::vector<uint32_t> id(hdr->has_ids ? n : 0);
    uint64_t sum = 0;
    if ((n && (std::fread(p.data(), sizeof(float4), n, fh.f) != n || std::fread(v.data(), sizeof(float4), n, fh.f) != n)) ||
        (hdr->has_ids && n && std::fread(id.data(), sizeof(uint32_t), n, fh.f) != n) ||
        std::fread(&sum, sizeof sum, 1, fh.f) != 1)
        return fail(WC_ERR_INVALID_ARG, "snapshot '%s' is truncated", path);
    char extra;
    if (std::fread(&extra, 1, 1, fh.f) != 0) return fail(WC_ERR_INVALID_ARG, "snapshot '%s' has trailing bytes", path);
    uint64_t h = fnv1a(FNV_OFFSET, hdr, sizeof *hdr);
    h = fnv1a(h, p.data(), sizeof(float4) * n);
    h = fnv1a(h, v.data(), sizeof(float4) * n);
    if (hdr->has_ids) h = fnv1a(h, id.data(), sizeof(uint32_t) * n);
    if (h != sum) return fail(WC_ERR_INVALID_ARG, "snapshot '%s' fails its checksum", path);
    if (pos) pos->swap(p);
    if (vel) vel->swap(v);
    if (ids) ids->swap(id);
    return WC_OK;
}

}  // namespace

extern "C" {

WC_API wc_status wc_fluid_save_snapshot(wc_fluid* f, const char* path, uint64_t seed) {
    clear_error();
    WC_NVTX("wc_fluid_save_snapshot");
    if (!f || !path) return fail(WC_ERR_INVALID_ARG, "null argument");
    WC_TRY(wc_fluid_synchronize(f));
    FluidInternals fi = fluid_internals(f);
    const DevBuffers& d = *fi.d;
    const size_t n = d.n;
    wc_snapshot_header hdr;
    std::memset(&hdr, 0, sizeof hdr);
    std::memcpy(hdr.magic, MAGIC, sizeof MAGIC);
    hdr.version = VERSION;
    hdr.header_bytes = sizeof hdr;
    hdr.num_particles = n;
    hdr.step = wc_fluid_step_count(f);
    hdr.seed = seed;
    hdr.has_ids = d.ids_a ? 1u : 0u;
    hdr.params = *fi.params;
    for (int a = 0; a < 3; ++a) {
        hdr.params.gravity[a] = fi.in->g[a];
        hdr.params.mouse_origin[a] = fi.in->mouse_o[a];
        hdr.params.mouse_dir[a] = fi.in->mouse_d[a];
    }
    std::vector<float4> p(n), v(n);
    std::vector<uint32_t> id(hdr.has_ids ? n : 0);
    if (n) {
        WC_CUDA_TRY(cudaMemcpyAsync(p.data(), d.pos_a, sizeof(float4) * n, cudaMemcpyDeviceToHost, fi.stream));
        WC_CUDA_TRY(cudaMemcpyAsync(v.data(), d.vel_a, sizeof(float4) * n, cudaMemcpyDeviceToHost, fi.stream));
        if (hdr.has_ids)
            WC_CUDA_TRY(cudaMemcpyAsync(id.data(), d.ids_a, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, fi.stream));
        WC_CUDA_TRY(cudaStreamSynchronize(fi.stream));
    }
    uint64_t h = fnv1a(FNV_OFFSET, &hdr, sizeof hdr);
    h = fnv1a(h, p.data(), sizeof(float4) * n);
    h = fnv1a(h, v.data(), sizeof(float4) * n);
    if (hdr.has_ids) h = fnv1a(h, id.data(), sizeof(uint32_t) * n);
    File fh;
    fh.f = std::fopen(path, "wb");
    if (!fh.f) return fail(WC_ERR_INVALID_ARG, "cannot create snapshot '%s'", path);
    bool ok = std::fwrite(&hdr, sizeof hdr, 1, fh.f) == 1;
    ok = ok && (!n || std::fwrite(p.data(), sizeof(float4), n, fh.f) == n);
    ok = ok && (!n || std::fwrite(v.data(), sizeof(float4), n, fh.f) == n);
    ok = ok && (!hdr.has_ids || !n || std::fwrite(id.data(), sizeof(uint32_t), n, fh.f) == n);
    ok = ok && std::fwrite(&h, sizeof h, 1, fh.f) == 1;
    ok = (std::fclose(fh.f) == 0) && ok;
    fh.f = nullptr;
    if (!ok) return fail(WC_ERR_INVALID_ARG, "writing snapshot '%s' failed", path);
    return WC_OK;
}

WC_API wc_status wc_snapshot_read_header(const char* path, wc_snapshot_header* out) {
    clear_error();
    return read_file(path, out, nullptr, nullptr, nullptr);
}

WC_API wc_status wc_fluid_load_snapshot(wc_fluid* f, const char* path) {
    clear_error();
    WC_NVTX("wc_fluid_load_snapshot");
    if (!f) return fail(WC_ERR_INVALID_ARG, "null fluid");
    wc_snapshot_header hdr;
    std::vector<float4> p, v;
    std::vector<uint32_t> id;
    WC_TRY(read_file(path, &hdr, &p, &v, &id));
    wc_params mine;
    WC_TRY(wc_fluid_get_params(f, &mine));
    if (!same_fixed_params(hdr.params, mine))
        return fail(WC_ERR_INVALID_ARG, "snapshot '%s' was saved with other parameters than this fluid's", path);
    FluidInternals fi = fluid_internals(f);
    DevBuffers& d = *fi.d;
    if (hdr.has_ids != (d.ids_a ? 1u : 0u))
        return fail(WC_ERR_INVALID_ARG, "snapshot '%s' %s particle ids; this fluid %s", path,
                    hdr.has_ids ? "carries" : "has no", d.ids_a ? "tracks them" : "does not");
    WC_TRY(wc_fluid_set_gravity(f, hdr.params.gravity));
    WC_TRY(wc_fluid_set_mouse_ray(f, hdr.params.mouse_origin, hdr.params.mouse_dir));
    WC_CUDA_TRY(cudaStreamSynchronize(fi.stream));
    const size_t n = d.n;
    if (n) {
        WC_CUDA_TRY(cudaMemcpy(d.pos_a, p.data(), sizeof(float4) * n, cudaMemcpyHostToDevice));
        WC_CUDA_TRY(cudaMemcpy(d.vel_a, v.data(), sizeof(float4) * n, cudaMemcpyHostToDevice));
        if (hdr.has_ids) WC_CUDA_TRY(cudaMemcpy(d.ids_a, id.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice));
    }
    fluid_set_step_count(f, hdr.step);
    return WC_OK;
}

WC_API wc_status wc_fluid_create_from_snapshot(const char* path, wc_fluid** out) {
    clear_error();
    if (!out) return fail(WC_ERR_INVALID_ARG, "null output");
    *out = nullptr;
    wc_snapshot_header hdr;
    WC_TRY(read_file(path, &hdr, nullptr, nullptr, nullptr));
    wc_fluid* f = nullptr;
    WC_TRY(wc_fluid_create(&hdr.params, &f));
    // setup marks the handle ready; the snapshot then overwrites the state
    std::vector<wc_particle> zero(hdr.num_particles);
    std::memset(zero.data(), 0, sizeof(wc_particle) * zero.size());
    for (size_t i = 0; i < zero.size(); ++i)
        for (int a = 0; a < 3; ++a) zero[i].position[a] = 0.5f * hdr.params.size;
    wc_status st = wc_fluid_setup(f, zero.data(), (uint32_t)hdr.num_particles);
    if (st == WC_OK) st = wc_fluid_load_snapshot(f, path);
    if (st != WC_OK) {
        wc_fluid_destroy(f);
        return st;
    }
    *out = f;
    return WC_OK;
}

}  // extern "C"
