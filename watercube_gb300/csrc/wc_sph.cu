// wc_sph.cu — the two neighbour passes of a step, as persistent sm_103a kernels.
//
//   density_kernel  density.comp:81-137  Poly6 density + equation of state (+ the reference's
//                                        wall pseudo-density when enabled)
//   force_kernel    update.comp:134-232  Spiky pressure + Laplacian viscosity + gravity (+ wall
//                                        and mouse forces), fused with symplectic Euler and the
//                                        box-wall collision
//
// Work decomposition (both kernels): a warp owns one non-empty cell at a time (grid-stride over
// the cell list the scan produced). The 27 neighbour cells of a cell form 9 rows of 3 cells
// that are contiguous in key order, hence 9 contiguous ranges of the sorted particle buffer;
// lanes 0..8 look them up once per cell. The warp's 32 lanes are split into nt targets (the
// cell's particles, up to 32 at a time) x S = floor(32/nt) slices; slice s of target t tests
// candidates s, s+S, s+2S, ... of every row, so every lane of the warp runs the same trip count
// and each candidate load is shared by the nt lanes that need it. Partial sums are combined
// with shuffles in a fixed order: results are deterministic.
//
// Neighbour test: |r| < h is evaluated exactly as sqrtf(fma(dz,dz,fma(dy,dy,dx*dx))) < h would
// be, as d2 <= cull with cull = the largest float whose sqrtf is below h, so the neighbour
// sets (and counts) are bit-identical to the reference stage logic's.
#include <cuda_runtime.h>

#include "wc_internal.h"

namespace wc {
namespace {

constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ float dist2(float dx, float dy, float dz) {
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

// Lanes 0..8 of the warp get the sorted-slot range [lo, hi) of neighbour row (dy, dz) of cell
// (cx, cy, cz); other lanes (and rows outside the grid) get an empty range.
__device__ __forceinline__ void row_range(const uint32_t* __restrict__ start, uint32_t n, int32_t R, int cx, int cy,
                                          int cz, uint32_t lane, uint32_t& lo, uint32_t& hi) {
    lo = hi = 0u;
    if (lane < 9u) {
        const int yy = cy + (int)(lane % 3u) - 1;
        const int zz = cz + (int)(lane / 3u) - 1;
        if (yy >= 0 && yy < R && zz >= 0 && zz < R) {
            const int x0 = cx > 0 ? cx - 1 : 0;
            const int x1 = cx + 1 < R ? cx + 1 : R - 1;
            const uint32_t row = (uint32_t)((zz * R + yy) * R);
            lo = __ldg(start + row + x0);
            hi = __ldg(start + row + x1 + 1);
            // Only a timed-out scan (reported as an error) leaves inconsistent tables; keep
            // the ranges inside the particle buffer regardless.
            hi = min(hi, n);
            lo = min(lo, hi);
        }
    }
}

// Sum v over the S slices of each target (lanes t + s*nt); the total lands in slice 0.
template <class T>
__device__ __forceinline__ T slice_sum(T v, uint32_t S, uint32_t nt, uint32_t sl) {
    for (uint32_t len = S; len > 1u;) {
        const uint32_t half = (len + 1u) >> 1;
        const T o = __shfl_down_sync(FULL, v, half * nt);
        if (sl + half < len) v += o;
        len = half;
    }
    return v;
}

// density.comp:53-55 evaluated as the reference does, for the wall term.
__device__ __forceinline__ float poly6_ref(const SceneConsts& c, float r) {
    const float w = c.h * c.h - r * r;
    return w * w * w * c.c6;
}

// density.comp:57-79, including its z branch that tests p.y.
__device__ float wall_density(const SceneConsts& c, float x, float y, float z) {
    float d = 0.f;
    if (x < c.h) d += c.m * poly6_ref(c, x);
    else if (x > c.size - c.h) d += c.m * poly6_ref(c, c.size - x);
    if (y < c.h) d += c.m * poly6_ref(c, y);
    else if (y > c.size - c.h) d += c.m * poly6_ref(c, c.size - y);
    if (z < c.h) d += c.m * poly6_ref(c, z);
    else if (y > c.size - c.h) d += c.m * poly6_ref(c, c.size - z);
    return d * 4.f;
}

// update.comp:71-100. The shader passes r.length() — the component count 3 — as the distance.
__device__ void wall_forces(const SceneConsts& c, const float p[3], float f[3]) {
    f[0] = f[1] = f[2] = 0.f;
    const float s = (c.h - 3.f) * (c.h - 3.f);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float target;
        bool hit = false;
        if (p[a] < c.h) { target = 0.f; hit = true; }
        else if (p[a] > c.size - c.h) { target = c.size; hit = true; }
        if (hit) f[a] += (s * ((target - p[a]) / 3.f)) * c.cs;  // r has only its a-component
    }
    f[0] *= 0.01f; f[1] *= 0.01f; f[2] *= 0.01f;
}

// update.comp:105-132 (slab test, then repulsion within h of the mouse ray).
__device__ void mouse_force(const SceneConsts& c, const StepInputs& in, const float p[3], float pressure,
                            float f[3]) {
    f[0] = f[1] = f[2] = 0.f;
    float t1[3], t2[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float tmin = (0.f - in.mouse_o[a]) / in.mouse_d[a];
        const float tmax = (c.size - in.mouse_o[a]) / in.mouse_d[a];
        t1[a] = tmax < tmin ? tmax : tmin;
        t2[a] = tmin < tmax ? tmax : tmin;
    }
    float tnear = t1[0] < t1[1] ? t1[1] : t1[0];
    tnear = tnear < t1[2] ? t1[2] : tnear;
    float tfar = t2[1] < t2[0] ? t2[1] : t2[0];
    tfar = t2[2] < tfar ? t2[2] : tfar;
    if (tnear > tfar) return;
    const float* d = in.mouse_d;
    const float tm[3] = {p[0] - in.mouse_o[0], p[1] - in.mouse_o[1], p[2] - in.mouse_o[2]};
    const float cx = d[1] * tm[2] - tm[1] * d[2];
    const float cy = d[2] * tm[0] - tm[2] * d[0];
    const float cz = d[0] * tm[1] - tm[0] * d[1];
    const float dist = sqrtf(dist2(cx, cy, cz));
    if (dist > c.h) return;
    const float dd = dist + 1e-16f;
    const float s = (c.h - dd) * (c.h - dd);
    const float k = (-c.m * pressure) * 0.00001f;
#pragma unroll
    for (int a = 0; a < 3; ++a) f[a] = (k * ((s * (tm[a] / dd)) * c.cs));
}

__global__ void __launch_bounds__(SPH_THREADS) density_kernel(const SceneConsts sc, const uint32_t n,
                                                              const float4* __restrict__ pos_in,
                                                              float* rho_out,  // aliases pos_in[].w
                                                              float* p_out,    // aliases vel[].w
                                                              const uint32_t* __restrict__ start,
                                                              const uint32_t* __restrict__ cell_list,
                                                              const uint32_t* __restrict__ num_nonempty,
                                                              uint32_t* __restrict__ ncount) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t M = min(*num_nonempty, (uint32_t)sc.R * (uint32_t)sc.R * (uint32_t)sc.R);
    const int32_t R = sc.R;
    for (uint32_t m = warp; m < M; m += nwarps) {
        const uint32_t c = __ldg(cell_list + m);
        const uint32_t cend = min(__ldg(start + c + 1), n), cbeg = min(__ldg(start + c), cend);
        const int cx = (int)(c % (uint32_t)R), cy = (int)((c / (uint32_t)R) % (uint32_t)R),
                  cz = (int)(c / ((uint32_t)R * R));
        uint32_t rlo, rhi;
        row_range(start, n, R, cx, cy, cz, lane, rlo, rhi);
        for (uint32_t t0 = cbeg; t0 < cend; t0 += 32u) {
            const uint32_t nt = min(32u, cend - t0);
            const uint32_t S = 32u / nt;
            const uint32_t t = lane % nt, sl = lane / nt;
            const bool active = sl < S;
            const uint32_t ti = t0 + t;
            const float4 pi = pos_in[ti];
            float sum = 0.f;
            uint32_t cnt = 0;
#pragma unroll 1
            for (int r = 0; r < 9; ++r) {
                const uint32_t lo = __shfl_sync(FULL, rlo, r), hi = __shfl_sync(FULL, rhi, r);
                if (!active) continue;
#pragma unroll 4
                for (uint32_t k = lo + sl; k < hi; k += S) {
                    const float4 pj = __ldg(pos_in + k);
                    const float d2 = dist2(pi.x - pj.x, pi.y - pj.y, pi.z - pj.z);
                    if (d2 <= sc.cull) {
                        const float w = sc.h2 - d2;
                        sum = fmaf(w * w, w, sum);
                        ++cnt;
                    }
                }
            }
            sum = slice_sum(sum, S, nt, sl);
            cnt = slice_sum(cnt, S, nt, sl);
            if (sl == 0u) {
                // The sum includes the particle itself (w = h^2): the reference's m*W(0) term.
                const float rho = (sc.m * sc.c6) * sum;
                float pressure;
                if (sc.eos == WC_EOS_LINEAR) {
                    pressure = sc.p0 + sc.k * (rho - sc.rho0);
                } else {
                    const float x = rho / sc.rho0;
                    pressure = sc.p0 + sc.k * (x * x * x - 1.f);
                }
                float total = rho;
                if (sc.flags & WC_FLAG_WALL_DENSITY) total = rho + wall_density(sc, pi.x, pi.y, pi.z);
                rho_out[4 * (size_t)ti] = total;
                p_out[4 * (size_t)ti] = pressure;
                if (ncount) ncount[ti] = cnt - 1u;
            }
        }
    }
}

template <int CAP>
__device__ __forceinline__ void accumulate_list(const uint32_t* list, uint32_t cnt, uint32_t lane, const float4& pi,
                                                const float4& vi, const float4* __restrict__ pos,
                                                const float4* __restrict__ vel, float h, float f[6]) {
    for (uint32_t e = 0; e < cnt; ++e) {
        const uint32_t k = list[e * 32u + lane];
        const float4 pj = __ldg(pos + k);
        const float4 vj = __ldg(vel + k);
        const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
        const float d2 = dist2(rx, ry, rz);
        const float rsq = d2 > 0.f ? rsqrtf(d2) : 0.f;  // coincident pair: r = 0, no pressure push
        const float d = d2 * rsq;
        const float inv_rho = __frcp_rn(pj.w);
        const float hd = h - d;
        const float pres = (vi.w + vj.w) * (0.5f * inv_rho);  // (p_i + p_j) / (2 rho_j)
        if (pres > 0.f) {
            const float coef = pres * hd * hd * rsq;
            f[0] = fmaf(coef, rx, f[0]);
            f[1] = fmaf(coef, ry, f[1]);
            f[2] = fmaf(coef, rz, f[2]);
        }
        const float wv = hd * inv_rho;
        f[3] = fmaf(vj.x - vi.x, wv, f[3]);
        f[4] = fmaf(vj.y - vi.y, wv, f[4]);
        f[5] = fmaf(vj.z - vi.z, wv, f[5]);
    }
}

template <int CAP>
__global__ void __launch_bounds__(SPH_THREADS) force_kernel(const SceneConsts sc, const StepInputs in, const uint32_t n,
                                                            const float4* __restrict__ pos_b,
                                                            const float4* __restrict__ vel_b,
                                                            const uint32_t* __restrict__ ids_b,
                                                            float4* __restrict__ pos_a, float4* __restrict__ vel_a,
                                                            uint32_t* __restrict__ ids_a,
                                                            const uint32_t* __restrict__ start,
                                                            const uint32_t* __restrict__ cell_list,
                                                            const uint32_t* __restrict__ num_nonempty) {
    extern __shared__ uint32_t s_lists[];
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t* list = s_lists + (threadIdx.x >> 5) * (CAP * 32);
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t M = min(*num_nonempty, (uint32_t)sc.R * (uint32_t)sc.R * (uint32_t)sc.R);
    const int32_t R = sc.R;
    const float fp_scale = -sc.m * sc.cs;           // -m * spiky const
    const float fv_scale = sc.m * sc.cv * sc.mu;    // m * visc const * mu
    for (uint32_t m = warp; m < M; m += nwarps) {
        const uint32_t c = __ldg(cell_list + m);
        const uint32_t cend = min(__ldg(start + c + 1), n), cbeg = min(__ldg(start + c), cend);
        const int cx = (int)(c % (uint32_t)R), cy = (int)((c / (uint32_t)R) % (uint32_t)R),
                  cz = (int)(c / ((uint32_t)R * R));
        uint32_t rlo, rhi;
        row_range(start, n, R, cx, cy, cz, lane, rlo, rhi);
        for (uint32_t t0 = cbeg; t0 < cend; t0 += 32u) {
            const uint32_t nt = min(32u, cend - t0);
            const uint32_t S = 32u / nt;
            const uint32_t t = lane % nt, sl = lane / nt;
            const bool active = sl < S;
            const uint32_t ti = t0 + t;
            const float4 pi = pos_b[ti];
            const float4 vi = vel_b[ti];
            float f[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            uint32_t cnt = 0;
#pragma unroll 1
            for (int r = 0; r < 9; ++r) {
                const uint32_t lo = __shfl_sync(FULL, rlo, r), hi = __shfl_sync(FULL, rhi, r);
                const uint32_t iters = (hi - lo + S - 1u) / S;
                for (uint32_t seg = 0; seg < iters; seg += CAP) {
                    const uint32_t seg_iters = min((uint32_t)CAP, iters - seg);
                    if (__any_sync(FULL, cnt + seg_iters > (uint32_t)CAP)) {
                        accumulate_list<CAP>(list, cnt, lane, pi, vi, pos_b, vel_b, sc.h, f);
                        cnt = 0;
                    }
                    if (active) {
                        const uint32_t k0 = lo + seg * S + sl;
#pragma unroll 4
                        for (uint32_t it = 0; it < seg_iters; ++it) {
                            const uint32_t k = k0 + it * S;
                            if (k < hi) {
                                const float4 pj = __ldg(pos_b + k);
                                const float d2 = dist2(pi.x - pj.x, pi.y - pj.y, pi.z - pj.z);
                                // The particle itself passes too; it contributes exactly zero.
                                if (d2 <= sc.cull) list[(cnt++) * 32u + lane] = k;
                            }
                        }
                    }
                }
            }
            accumulate_list<CAP>(list, cnt, lane, pi, vi, pos_b, vel_b, sc.h, f);
#pragma unroll
            for (int q = 0; q < 6; ++q) f[q] = slice_sum(f[q], S, nt, sl);
            if (sl == 0u) {
                const float rho = pi.w, pressure = vi.w;
                const float p3[3] = {pi.x, pi.y, pi.z};
                float ext[3] = {in.g[0] * rho, in.g[1] * rho, in.g[2] * rho};
                if (sc.flags & (WC_FLAG_WALL_FORCE | WC_FLAG_MOUSE_FORCE)) {
                    float wf[3] = {0.f, 0.f, 0.f}, mf[3] = {0.f, 0.f, 0.f};
                    if (sc.flags & WC_FLAG_WALL_FORCE) wall_forces(sc, p3, wf);
                    if (sc.flags & WC_FLAG_MOUSE_FORCE) mouse_force(sc, in, p3, pressure, mf);
#pragma unroll
                    for (int a = 0; a < 3; ++a) ext[a] += mf[a] + wf[a];
                }
                const float inv = 1.f / (rho + 1e-16f);
                const float vin[3] = {vi.x, vi.y, vi.z};
                float v[3], x[3];
#pragma unroll
                for (int a = 0; a < 3; ++a) {
                    const float force = fp_scale * f[a] + fv_scale * f[3 + a] + ext[a];
                    float va = vin[a] + (force * inv) * in.dt;
                    if (sc.flags & WC_FLAG_SPEED_CLAMP) va = fminf(fmaxf(va, -sc.max_speed), sc.max_speed);
                    float xa = p3[a] + va * in.dt;
                    if (xa < sc.border) {
                        va *= -sc.damping;
                        xa = sc.border;
                    } else if (xa > sc.size - sc.border) {
                        va *= -sc.damping;
                        xa = sc.size - sc.border;
                    }
                    v[a] = va;
                    x[a] = xa;
                }
                pos_a[ti] = make_float4(x[0], x[1], x[2], rho);
                vel_a[ti] = make_float4(v[0], v[1], v[2], pressure);
                if (ids_a) ids_a[ti] = ids_b[ti];
            }
        }
    }
}

constexpr size_t force_smem_bytes() { return (size_t)(SPH_THREADS / 32) * FORCE_LIST_CAP * 32 * sizeof(uint32_t); }

}  // namespace

LaunchDims compute_launch_dims(int device) {
    LaunchDims ld;
    cudaDeviceGetAttribute(&ld.sms, cudaDevAttrMultiProcessorCount, device);
    if (ld.sms <= 0) ld.sms = 1;
    int bd = 0, bf = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bd, density_kernel, SPH_THREADS, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bf, force_kernel<FORCE_LIST_CAP>, SPH_THREADS, force_smem_bytes());
    ld.grid_density = ld.sms * (bd > 0 ? bd : 1);
    ld.grid_force = ld.sms * (bf > 0 ? bf : 1);
    ld.grid_stream = ld.sms * 8;
    return ld;
}

void launch_density(const DevBuffers& d, const SceneConsts& sc, const LaunchDims& ld, cudaStream_t s) {
    density_kernel<<<ld.grid_density, SPH_THREADS, 0, s>>>(
        sc, d.n, d.pos_b, reinterpret_cast<float*>(d.pos_b) + 3, reinterpret_cast<float*>(d.vel_b) + 3, d.start,
        d.cell_list, d.num_nonempty, (sc.flags & WC_FLAG_NEIGHBOR_COUNTS) ? d.ncount : nullptr);
}

void launch_force(const DevBuffers& d, const SceneConsts& sc, const StepInputs& in, const LaunchDims& ld,
                  cudaStream_t s) {
    force_kernel<FORCE_LIST_CAP><<<ld.grid_force, SPH_THREADS, force_smem_bytes(), s>>>(
        sc, in, d.n, d.pos_b, d.vel_b, d.ids_b, d.pos_a, d.vel_a, d.ids_a, d.start, d.cell_list, d.num_nonempty);
}

const void* force_kernel_symbol(uint32_t) { return reinterpret_cast<const void*>(&force_kernel<FORCE_LIST_CAP>); }

}  // namespace wc
