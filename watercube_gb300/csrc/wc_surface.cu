// wc_surface.cu — surface extraction from the particles: a colour field on a vertex grid and
// marching cubes over it (no counterpart in the reference, which draws the particles as
// points; surface reconstruction is its report's stated future work).
//
//   field      phi(v) = sum_j (m / rho0) W_poly6(|v - x_j|, h) over the particles of the 27 cells
//              around vertex v (the solver's sorted buffer and cell tables), about 1 inside the
//              fluid and 0 outside; every float operation is an explicit round-to-nearest one,
//              summed in the cell-row order of the tables, so the result is reproducible exactly
//   classify   per cube: corner bits (phi > iso), triangle count from the case table
//   scan       the decoupled look-back scan of the solver over the per-cube counts
//   emit       per cube: its triangles, each vertex interpolated on a cube edge whose
//              endpoints are taken in ascending order (neighbouring cubes produce the same
//              float coordinates, so the mesh is watertight)
//
// The case table is generated here, not typed in: for each of the 256 corner configurations
// the iso-segments of the six faces are walked (on a face with two diagonal inside corners the
// segments separate the inside corners; the decision depends only on the face, so both cubes
// sharing it agree), chained into closed loops, oriented so that the normal (Newell's method)
// points from the inside corners to the outside ones, and triangulated as fans.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "wc_internal.h"
#include "wc_util.h"

using namespace wc;

namespace {

constexpr int MAX_TRI = 12;  // per cube (a configuration yields at most 10)

// Corner c sits at offset (c & 1, (c >> 1) & 1, (c >> 2) & 1). Edge e joins corners
// EDGE_A[e] < EDGE_B[e], which differ in the bit of axis e / 4.
constexpr int EDGE_A[12] = {0, 2, 4, 6, 0, 1, 4, 5, 0, 1, 2, 3};
constexpr int EDGE_B[12] = {1, 3, 5, 7, 2, 3, 6, 7, 4, 5, 6, 7};

struct CaseTable {
    uint8_t count[256];
    int8_t tri[256][MAX_TRI * 3];
};

int edge_of(int a, int b) {
    if (a > b) std::swap(a, b);
    for (int e = 0; e < 12; ++e)
        if (EDGE_A[e] == a && EDGE_B[e] == b) return e;
    return -1;
}

void corner_pos(int c, double p[3]) {
    p[0] = c & 1;
    p[1] = (c >> 1) & 1;
    p[2] = (c >> 2) & 1;
}

// One configuration's triangles (edge triples).
void build_case(int cfg, std::vector<int>& tris) {
    tris.clear();
    auto inside = [&](int c) { return (cfg >> c) & 1; };
    std::vector<std::pair<int, int>> segs;  // undirected, between crossing edges
    for (int a = 0; a < 3; ++a) {
        const int u = (a + 1) % 3, v = (a + 2) % 3;
        for (int s = 0; s < 2; ++s) {
            // the face's corners in cyclic order (u, v) = (0,0), (1,0), (1,1), (0,1)
            int cyc[4];
            const int uv[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
            for (int k = 0; k < 4; ++k) cyc[k] = (s << a) | (uv[k][0] << u) | (uv[k][1] << v);
            int fe[4];
            bool cross[4];
            int ncross = 0;
            for (int k = 0; k < 4; ++k) {
                fe[k] = edge_of(cyc[k], cyc[(k + 1) & 3]);
                cross[k] = inside(cyc[k]) != inside(cyc[(k + 1) & 3]);
                ncross += cross[k];
            }
            if (ncross == 2) {
                int e0 = -1, e1 = -1;
                for (int k = 0; k < 4; ++k)
                    if (cross[k]) (e0 < 0 ? e0 : e1) = fe[k];
                segs.push_back({e0, e1});
            } else if (ncross == 4) {
                // two diagonal inside corners: cut each off on its own
                for (int k = 0; k < 4; ++k)
                    if (inside(cyc[k])) segs.push_back({fe[(k + 3) & 3], fe[k]});
            }
        }
    }
    // chain into loops (every crossing edge has exactly two segments)
    std::vector<bool> used(segs.size(), false);
    for (size_t first = 0; first < segs.size(); ++first) {
        if (used[first]) continue;
        std::vector<int> loop;
        used[first] = true;
        const int start = segs[first].first;
        int cur = segs[first].second;
        loop.push_back(start);
        while (cur != start) {
            loop.push_back(cur);
            bool found = false;
            for (size_t i = 0; i < segs.size(); ++i) {
                if (used[i]) continue;
                if (segs[i].first == cur || segs[i].second == cur) {
                    used[i] = true;
                    cur = segs[i].first == cur ? segs[i].second : segs[i].first;
                    found = true;
                    break;
                }
            }
            if (!found) break;  // cannot happen for a closed surface
        }
        // orientation: Newell normal of the loop (edge midpoints) against inside -> outside
        double nrm[3] = {0, 0, 0}, din[3] = {0, 0, 0}, dout[3] = {0, 0, 0};
        const size_t L = loop.size();
        std::vector<std::array<double, 3>> pts(L);
        for (size_t i = 0; i < L; ++i) {
            double pa[3], pb[3];
            corner_pos(EDGE_A[loop[i]], pa);
            corner_pos(EDGE_B[loop[i]], pb);
            for (int k = 0; k < 3; ++k) pts[i][k] = 0.5 * (pa[k] + pb[k]);
            const bool ain = inside(EDGE_A[loop[i]]);
            for (int k = 0; k < 3; ++k) {
                din[k] += ain ? pa[k] : pb[k];
                dout[k] += ain ? pb[k] : pa[k];
            }
        }
        for (size_t i = 0; i < L; ++i) {
            const auto& p = pts[i];
            const auto& q = pts[(i + 1) % L];
            nrm[0] += (p[1] - q[1]) * (p[2] + q[2]);
            nrm[1] += (p[2] - q[2]) * (p[0] + q[0]);
            nrm[2] += (p[0] - q[0]) * (p[1] + q[1]);
        }
        const double dot = nrm[0] * (dout[0] - din[0]) + nrm[1] * (dout[1] - din[1]) + nrm[2] * (dout[2] - din[2]);
        if (dot < 0) std::reverse(loop.begin() + 1, loop.end());
        for (size_t i = 1; i + 1 < L; ++i) {
            tris.push_back(loop[0]);
            tris.push_back(loop[i]);
            tris.push_back(loop[i + 1]);
        }
    }
}

const CaseTable& case_table() {
    static CaseTable t;
    static std::once_flag once;
    std::call_once(once, [] {
        std::memset(&t, 0, sizeof t);
        std::memset(t.tri, -1, sizeof t.tri);
        std::vector<int> tris;
        for (int cfg = 0; cfg < 256; ++cfg) {
            build_case(cfg, tris);
            const int nt = (int)tris.size() / 3;
            t.count[cfg] = (uint8_t)(nt > MAX_TRI ? MAX_TRI : nt);
            for (int i = 0; i < t.count[cfg] * 3; ++i) t.tri[cfg][i] = (int8_t)tris[i];
        }
    });
    return t;
}

__constant__ uint8_t c_count[256];
__constant__ int8_t c_tri[256][MAX_TRI * 3];
__constant__ int8_t c_edge_a[12];
__constant__ int8_t c_edge_b[12];

struct Grid {
    uint32_t G;     // vertices per axis
    float spacing;  // size / (G - 1)
};

__device__ __forceinline__ float vcoord(uint32_t i, float spacing) { return __fmul_rn((float)i, spacing); }

// phi at every vertex (x fastest). One thread per vertex.
__global__ void field_kernel(Grid g, const float4* __restrict__ pos, uint32_t n, const uint32_t* __restrict__ start,
                             float bin, int32_t R, float h2, float scale, float* __restrict__ phi,
                             uint32_t* __restrict__ err) {
    const uint64_t V = (uint64_t)g.G * g.G * g.G;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < V; v += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t ix = (uint32_t)(v % g.G), iy = (uint32_t)((v / g.G) % g.G), iz = (uint32_t)(v / ((uint64_t)g.G * g.G));
        const float px = vcoord(ix, g.spacing), py = vcoord(iy, g.spacing), pz = vcoord(iz, g.spacing);
        auto cell = [&](float q) {
            const float f = __fdiv_rn(q, bin);
            int c = f >= 1.0f ? (int)f : 0;
            return c > R - 1 ? R - 1 : c;
        };
        const int cx = cell(px), cy = cell(py), cz = cell(pz);
        float acc = 0.f;
        for (int dz = -1; dz <= 1; ++dz) {
            const int z = cz + dz;
            if (z < 0 || z >= R) continue;
            for (int dy = -1; dy <= 1; ++dy) {
                const int y = cy + dy;
                if (y < 0 || y >= R) continue;
                const int x0 = cx > 0 ? cx - 1 : 0, x1 = cx + 1 < R ? cx + 1 : R - 1;
                const uint32_t row = (uint32_t)((z * R + y) * R);
                const uint32_t hi = min(start[row + x1 + 1], n);
                const uint32_t lo = min(start[row + x0], hi);
                if (hi - lo > 3u * MAX_CELL_PARTICLES) {  // a collapsed state: not evaluated
                    acc = __int_as_float(0x7fc00000);
                    atomicOr(err, DEVERR_CELL_OVERFLOW);
                    continue;
                }
                for (uint32_t k = lo; k < hi; ++k) {
                    const float4 q = __ldg(pos + k);
                    const float dx = __fsub_rn(px, q.x), dyy = __fsub_rn(py, q.y), dzz = __fsub_rn(pz, q.z);
                    const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dyy, dyy)), __fmul_rn(dzz, dzz));
                    if (d2 < h2) {
                        const float t = __fsub_rn(h2, d2);
                        acc = __fadd_rn(acc, __fmul_rn(__fmul_rn(t, t), t));
                    }
                }
            }
        }
        phi[v] = __fmul_rn(acc, scale);
    }
}

__device__ __forceinline__ uint32_t cube_config(const float* __restrict__ phi, uint32_t G, uint32_t ix, uint32_t iy,
                                                uint32_t iz, float iso) {
    uint32_t cfg = 0;
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        const uint64_t idx = ((uint64_t)(iz + ((c >> 2) & 1)) * G + (iy + ((c >> 1) & 1))) * G + (ix + (c & 1));
        cfg |= (phi[idx] > iso ? 1u : 0u) << c;
    }
    return cfg;
}

__global__ void classify_kernel(uint32_t G, const float* __restrict__ phi, float iso, uint32_t* __restrict__ counts) {
    const uint32_t C = G - 1;
    const uint64_t cubes = (uint64_t)C * C * C;
    for (uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; q < cubes; q += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t ix = (uint32_t)(q % C), iy = (uint32_t)((q / C) % C), iz = (uint32_t)(q / ((uint64_t)C * C));
        counts[q] = c_count[cube_config(phi, G, ix, iy, iz, iso)];
    }
}

__global__ void emit_kernel(Grid g, const float* __restrict__ phi, float iso, const uint32_t* __restrict__ offsets,
                            uint64_t max_tris, float* __restrict__ out) {
    const uint32_t G = g.G, C = G - 1;
    const uint64_t cubes = (uint64_t)C * C * C;
    for (uint64_t q = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; q < cubes; q += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t ix = (uint32_t)(q % C), iy = (uint32_t)((q / C) % C), iz = (uint32_t)(q / ((uint64_t)C * C));
        const uint32_t cfg = cube_config(phi, G, ix, iy, iz, iso);
        const uint32_t nt = c_count[cfg];
        if (!nt) continue;
        const uint64_t base = offsets[q];
        for (uint32_t t = 0; t < nt; ++t) {
            if (base + t >= max_tris) return;  // (the host sizes the buffer from the scan total)
            float* o = out + (base + t) * 9u;
            for (int k = 0; k < 3; ++k) {
                const int e = c_tri[cfg][3 * t + k];
                const int a = c_edge_a[e], b = c_edge_b[e];
                const uint32_t ax = ix + (a & 1), ay = iy + ((a >> 1) & 1), az = iz + ((a >> 2) & 1);
                const uint32_t bx = ix + (b & 1), by = iy + ((b >> 1) & 1), bz = iz + ((b >> 2) & 1);
                const float fa = phi[((uint64_t)az * G + ay) * G + ax];
                const float fb = phi[((uint64_t)bz * G + by) * G + bx];
                const float s = __fdiv_rn(__fsub_rn(iso, fa), __fsub_rn(fb, fa));
                const float pa[3] = {vcoord(ax, g.spacing), vcoord(ay, g.spacing), vcoord(az, g.spacing)};
                const float pb[3] = {vcoord(bx, g.spacing), vcoord(by, g.spacing), vcoord(bz, g.spacing)};
#pragma unroll
                for (int d = 0; d < 3; ++d) o[3 * k + d] = __fadd_rn(pa[d], __fmul_rn(s, __fsub_rn(pb[d], pa[d])));
            }
        }
    }
}

template <class T>
wc_status dalloc(T** p, size_t count) {
    *p = nullptr;
    if (!count) return WC_OK;
    WC_TRY(::wc::device_alloc(reinterpret_cast<void**>(p), count * sizeof(T)));
    return WC_OK;
}

}  // namespace

struct wc_surface {
    wc_surface_params p{};
    uint32_t G = 0;
    float* phi = nullptr;
    uint32_t *counts = nullptr, *offsets = nullptr, *cell_list = nullptr, *words = nullptr, *err = nullptr;
    unsigned long long* desc = nullptr;
    float* tris = nullptr;
    uint64_t tri_cap = 0, ntris = 0;
    float spacing = 0.f, iso = 0.f;
    bool have = false;
    cudaStream_t stream = nullptr;
    float ms_field = 0.f, ms_mesh = 0.f;
};

namespace {

wc_status upload_tables() {
    static std::once_flag once;
    static cudaError_t rc = cudaSuccess;
    std::call_once(once, [] {
        const CaseTable& t = case_table();
        int8_t ea[12], eb[12];
        for (int e = 0; e < 12; ++e) {
            ea[e] = (int8_t)EDGE_A[e];
            eb[e] = (int8_t)EDGE_B[e];
        }
        rc = cudaMemcpyToSymbol(c_count, t.count, sizeof t.count);
        if (rc == cudaSuccess) rc = cudaMemcpyToSymbol(c_tri, t.tri, sizeof t.tri);
        if (rc == cudaSuccess) rc = cudaMemcpyToSymbol(c_edge_a, ea, sizeof ea);
        if (rc == cudaSuccess) rc = cudaMemcpyToSymbol(c_edge_b, eb, sizeof eb);
    });
    if (rc != cudaSuccess) return fail(WC_ERR_CUDA, "surface tables: %s", cudaGetErrorString(rc));
    return WC_OK;
}

unsigned grid_blocks(uint64_t work) {
    const uint64_t b = (work + 255) / 256;
    return (unsigned)(b > 152ull * 64 ? 152ull * 64 : (b ? b : 1));
}

}  // namespace

extern "C" {

WC_API wc_status wc_surface_case_table(uint8_t* counts, int8_t* tris) {
    clear_error();
    if (!counts || !tris) return fail(WC_ERR_INVALID_ARG, "null argument");
    const CaseTable& t = case_table();
    std::memcpy(counts, t.count, sizeof t.count);
    std::memcpy(tris, t.tri, sizeof t.tri);
    return WC_OK;
}

WC_API wc_status wc_surface_create(const wc_surface_params* p, wc_surface** out) {
    clear_error();
    if (!p || !out) return fail(WC_ERR_INVALID_ARG, "null argument");
    if (p->grid_res < 2 || p->grid_res > 1024) return fail(WC_ERR_INVALID_ARG, "grid_res must be in 2..1024");
    wc_surface* s = new (std::nothrow) wc_surface();
    if (!s) return fail(WC_ERR_OOM, "host allocation failed");
    s->p = *p;
    s->G = p->grid_res;
    const uint64_t V = (uint64_t)s->G * s->G * s->G;
    const uint64_t C = (uint64_t)(s->G - 1) * (s->G - 1) * (s->G - 1);
    wc_status st = upload_tables();
    if (st == WC_OK && C > 0xffffffffull) st = fail(WC_ERR_INVALID_ARG, "too many cubes");
    if (st == WC_OK && cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess)
        st = fail(WC_ERR_CUDA, "stream creation failed");
    const uint64_t tiles = (C + SCAN_TILE - 1) / SCAN_TILE;
    if (st == WC_OK) st = dalloc(&s->phi, V);
    if (st == WC_OK) st = dalloc(&s->counts, C);
    if (st == WC_OK) st = dalloc(&s->offsets, C + 1);
    if (st == WC_OK) st = dalloc(&s->cell_list, C);
    if (st == WC_OK) st = dalloc(&s->words, 2);
    if (st == WC_OK) st = dalloc(&s->err, 1);
    if (st == WC_OK) st = dalloc(&s->desc, tiles ? tiles : 1);
    if (st == WC_OK && cudaMemset(s->err, 0, sizeof(uint32_t)) != cudaSuccess) st = fail(WC_ERR_CUDA, "memset");
    if (st != WC_OK) {
        wc_surface_destroy(s);
        return st;
    }
    *out = s;
    return WC_OK;
}

WC_API void wc_surface_destroy(wc_surface* s) {
    if (!s) return;
    if (s->stream) cudaStreamSynchronize(s->stream);
    void* ptrs[] = {s->phi, s->counts, s->offsets, s->cell_list, s->words, s->err, s->desc, s->tris};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

WC_API wc_status wc_surface_extract(wc_surface* s, wc_fluid* f, uint64_t* num_triangles) {
    clear_error();
    WC_NVTX("wc_surface_extract");
    if (!s || !f) return fail(WC_ERR_INVALID_ARG, "null argument");
    FluidInternals fi = fluid_internals(f);
    const DevBuffers& d = *fi.d;
    const SceneConsts& sc = *fi.sc;
    const float radius = s->p.radius > 0.f ? s->p.radius : sc.h;
    if (radius > sc.bin) return fail(WC_ERR_INVALID_ARG, "field radius %g exceeds the cell edge %g", radius, sc.bin);
    const uint32_t G = s->G, C = G - 1;
    const uint64_t V = (uint64_t)G * G * G, cubes = (uint64_t)C * C * C;
    Grid g{G, sc.size / (float)(G - 1)};
    s->spacing = g.spacing;
    s->iso = s->p.iso;
    const float h2 = radius * radius;
    // m / rho0 * 315 / (64 pi r^9), the Poly6 normalisation for the field radius (r^9 by
    // repeated double multiplication, reproducible everywhere)
    const double r1 = radius, r2 = r1 * r1, r4 = r2 * r2, r8 = r4 * r4;
    const double c6 = 315.0 / (64.0 * M_PI * (r8 * r1));
    const float scale = (float)((double)sc.m / (double)sc.rho0 * c6);
    // sort the fluid's state (its cell tables then describe the sorted buffer)
    WC_CUDA_TRY(cudaStreamSynchronize(s->stream));
    fluid_enqueue_sort(f);
    cudaEvent_t e0, e1, e2;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventCreate(&e2);
    cudaEventRecord(e0, fi.stream);
    field_kernel<<<grid_blocks(V), 256, 0, fi.stream>>>(g, d.pos_b, d.n, d.start, sc.bin, sc.R, h2, scale, s->phi,
                                                        s->err);
    cudaEventRecord(e1, fi.stream);
    classify_kernel<<<grid_blocks(cubes), 256, 0, fi.stream>>>(G, s->phi, s->p.iso, s->counts);
    DevBuffers sd{};
    sd.n = 0;
    sd.num_cells = (uint32_t)cubes;
    sd.num_tiles = (uint32_t)((cubes + SCAN_TILE - 1) / SCAN_TILE);
    sd.counts = s->counts;
    sd.start = s->offsets;
    sd.cell_list = s->cell_list;
    sd.num_nonempty = s->words + 1;
    sd.scan_desc = s->desc;
    sd.scan_tile_counter = s->words;
    sd.err = s->err;
    WC_CUDA_TRY(cudaMemsetAsync(s->desc, 0, sizeof(unsigned long long) * (sd.num_tiles ? sd.num_tiles : 1), fi.stream));
    WC_CUDA_TRY(cudaMemsetAsync(s->words, 0, sizeof(uint32_t), fi.stream));
    launch_scan_cells(sd, fi.stream);
    uint32_t total = 0, err = 0;
    WC_CUDA_TRY(cudaMemcpyAsync(&total, s->offsets + cubes, sizeof total, cudaMemcpyDeviceToHost, fi.stream));
    WC_CUDA_TRY(cudaMemcpyAsync(&err, s->err, sizeof err, cudaMemcpyDeviceToHost, fi.stream));
    WC_CUDA_TRY(cudaStreamSynchronize(fi.stream));
    if (err) {
        cudaMemset(s->err, 0, sizeof(uint32_t));
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaEventDestroy(e2);
        if (err & DEVERR_CELL_OVERFLOW)
            return fail(WC_ERR_NUMERIC, "a cell row held more than %u particles (a collapsed or non-finite state)",
                        3u * MAX_CELL_PARTICLES);
        return fail(WC_ERR_TIMEOUT, "surface scan look-back exceeded its wait limit");
    }
    wc_status st = WC_OK;
    if (total > s->tri_cap) {
        if (s->tris) cudaFree(s->tris);
        s->tris = nullptr;
        s->tri_cap = 0;
        st = dalloc(&s->tris, (size_t)total * 9u);
        if (st == WC_OK) s->tri_cap = total;
    }
    if (st == WC_OK && total)
        emit_kernel<<<grid_blocks(cubes), 256, 0, fi.stream>>>(g, s->phi, s->p.iso, s->offsets, s->tri_cap, s->tris);
    cudaEventRecord(e2, fi.stream);
    const cudaError_t ce = cudaStreamSynchronize(fi.stream);
    cudaEventElapsedTime(&s->ms_field, e0, e1);
    cudaEventElapsedTime(&s->ms_mesh, e1, e2);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(e2);
    if (st != WC_OK) return st;
    if (ce != cudaSuccess) return fail(WC_ERR_CUDA, "surface extraction: %s", cudaGetErrorString(ce));
    s->ntris = total;
    s->have = true;
    if (num_triangles) *num_triangles = total;
    return WC_OK;
}

WC_API wc_status wc_surface_get_triangles(wc_surface* s, float* out, uint64_t num_triangles) {
    clear_error();
    if (!s || (!out && num_triangles)) return fail(WC_ERR_INVALID_ARG, "null argument");
    if (!s->have) return fail(WC_ERR_STATE, "no surface extracted yet");
    if (num_triangles != s->ntris)
        return fail(WC_ERR_INVALID_ARG, "buffer holds %llu triangles, the surface has %llu",
                    (unsigned long long)num_triangles, (unsigned long long)s->ntris);
    if (num_triangles)
        WC_CUDA_TRY(cudaMemcpy(out, s->tris, sizeof(float) * 9u * (size_t)num_triangles, cudaMemcpyDeviceToHost));
    return WC_OK;
}

WC_API wc_status wc_surface_get_field(wc_surface* s, float* out, uint64_t count) {
    clear_error();
    if (!s || !out) return fail(WC_ERR_INVALID_ARG, "null argument");
    if (!s->have) return fail(WC_ERR_STATE, "no surface extracted yet");
    if (count != (uint64_t)s->G * s->G * s->G) return fail(WC_ERR_INVALID_ARG, "field has grid_res^3 values");
    WC_CUDA_TRY(cudaMemcpy(out, s->phi, sizeof(float) * (size_t)count, cudaMemcpyDeviceToHost));
    return WC_OK;
}

WC_API wc_status wc_surface_timings(const wc_surface* s, float* ms_field, float* ms_mesh) {
    clear_error();
    if (!s) return fail(WC_ERR_INVALID_ARG, "null surface");
    if (ms_field) *ms_field = s->ms_field;
    if (ms_mesh) *ms_mesh = s->ms_mesh;
    return WC_OK;
}

}  // extern "C"
