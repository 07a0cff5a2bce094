// wc_sph.cu — the two neighbour passes of a step, as persistent sm_103a kernels.
//
//   density_kernel  density.comp:81-137  Poly6 density + equation of state (+ the reference's
//                                        wall pseudo-density when enabled)
//   force_kernel    update.comp:134-232  Spiky pressure + Laplacian viscosity + gravity (+ wall
//                                        and mouse forces), fused with symplectic Euler and the
//                                        box-wall collision
//
// Work decomposition (both kernels): a warp owns one non-empty cell at a time, taking the next
// index into the cell list the scan produced from a counter (dynamic scheduling). The 27 neighbour cells of a cell form 9 rows of 3 cells
// that are contiguous in key order, hence 9 contiguous ranges of the sorted particle buffer;
// lanes 0..8 look them up once per cell and a 9-lane scan numbers the concatenated candidate
// list 0 .. L-1. The warp's 32 lanes are split into nt targets (the cell's particles, up to 32
// at a time) x S = floor(32/nt) slices; slice s of target t takes candidate pairs s, s+S, ...,
// so every lane runs the same trip count. Partial sums are combined with shuffles in a fixed
// order: results are deterministic.
//
// Density: the candidates' positions are staged in shared memory as x/y/z arrays by
// asynchronous copies (cp.async: every row in flight at once, one wait) and tested four at a
// time with Blackwell's packed f32x2 arithmetic (one 128-bit shared load yields two packed
// pairs; one instruction updates two candidates). Each lane records which of its candidates
// passed as a bit string. The force pass decodes those bits once per cell into one neighbour
// list per target (shared memory, prefix sums over the target's slices), and the target's
// slices then split its list evenly, gathering four neighbours per round, instead of testing
// all candidates again. Compressed states outgrow that form: a candidate list longer than the
// stage streams through it in pieces (dense path), and a cell of more than 32 particles is
// taken 32 targets at a time. Their bit strings are kept whenever a chunk's words fit the
// per-particle slot (bits_fit), in pieces whole words long, and the force pass replays them
// piece by piece through slot tables into per-lane lists; where they are not kept, the force
// pass culls the candidates itself with the same packed test through a small stage.
//
// Neighbour test: |r| < h is evaluated exactly as sqrtf(fma(dz,dz,fma(dy,dy,dx*dx))) < h would
// be, as d2 <= cull with cull = the largest float whose sqrtf is below h, so the neighbour
// sets (and counts) are bit-identical to the reference stage logic's. The packed form computes
// the same fused operations per element, so it agrees bit for bit.
#include <cuda_runtime.h>

#include "wc_internal.h"

namespace wc {
namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr int WARPS = SPH_THREADS / 32;
// Force pass, dense path: candidates staged per piece, and the most slices a target takes.
constexpr int FORCE_STAGE = 128;
constexpr uint32_t FORCE_DENSE_SLICES = 4;
// Force pass, replay path: neighbour-list entries per warp (the dense path's list and stage space).
constexpr int FORCE_REPLAY_LIST = FORCE_LIST_CAP * 32 + 3 * FORCE_STAGE;
// Force pass, piecewise replay: per-lane list capacity (the same space split by lane).
constexpr int REPLAY_LANE_CAP = FORCE_REPLAY_LIST / 32;

// ---- packed f32x2 arithmetic (two floats in one 64-bit register; lo = first) ---------------------
typedef unsigned long long f2;
__device__ __forceinline__ f2 pk(float a, float b) {
    f2 r;
    asm("mov.b64 %0, {%1,%2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void upk(f2 v, float& a, float& b) { asm("mov.b64 {%0,%1}, %2;" : "=f"(a), "=f"(b) : "l"(v)); }
__device__ __forceinline__ f2 sub2(f2 a, f2 b) {
    f2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 mul2(f2 a, f2 b) {
    f2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
    f2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

__device__ __forceinline__ float dist2(float dx, float dy, float dz) {
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

// Four staged candidates against one target: hit bits (bit c for candidate c) and the Poly6
// weights (cull - d2)^3 of the hits added to acc01 / acc23. The stage holds CAP x values, then
// CAP y values, then CAP z values.
template <int CAP = STAGE_CAP>
__device__ __forceinline__ uint32_t quad_hits(const ulonglong2* q, f2 px, f2 py, f2 pz, f2 cull2, f2& acc01,
                                              f2& acc23) {
    const ulonglong2 X = q[0], Y = q[CAP / 4], Z = q[CAP / 2];
    const f2 dx01 = sub2(px, X.x), dx23 = sub2(px, X.y);
    const f2 dy01 = sub2(py, Y.x), dy23 = sub2(py, Y.y);
    const f2 dz01 = sub2(pz, Z.x), dz23 = sub2(pz, Z.y);
    const f2 d01 = fma2(dz01, dz01, fma2(dy01, dy01, mul2(dx01, dx01)));
    const f2 d23 = fma2(dz23, dz23, fma2(dy23, dy23, mul2(dx23, dx23)));
    // u = cull - d2 >= 0 exactly when d2 <= cull (a tie gives +0): the sign bits are the misses.
    float u0, u1, u2, u3;
    upk(sub2(cull2, d01), u0, u1);
    upk(sub2(cull2, d23), u2, u3);
    const uint32_t miss = (__float_as_uint(u0) >> 31) | ((__float_as_uint(u1) >> 30) & 2u) |
                          ((__float_as_uint(u2) >> 29) & 4u) | ((__float_as_uint(u3) >> 28) & 8u);
    // Poly6 weight (cull - d2)^3 for hits, 0 otherwise (cull is h^2 to the ulp).
    const f2 w01 = pk(fmaxf(u0, 0.f), fmaxf(u1, 0.f));
    const f2 w23 = pk(fmaxf(u2, 0.f), fmaxf(u3, 0.f));
    acc01 = fma2(mul2(w01, w01), w01, acc01);
    acc23 = fma2(mul2(w23, w23), w23, acc23);
    return miss ^ 0xFu;
}

// The same test without the weights (the force pass's culling).
template <int CAP>
__device__ __forceinline__ uint32_t quad_test(const ulonglong2* q, f2 px, f2 py, f2 pz, f2 cull2) {
    const ulonglong2 X = q[0], Y = q[CAP / 4], Z = q[CAP / 2];
    const f2 dx01 = sub2(px, X.x), dx23 = sub2(px, X.y);
    const f2 dy01 = sub2(py, Y.x), dy23 = sub2(py, Y.y);
    const f2 dz01 = sub2(pz, Z.x), dz23 = sub2(pz, Z.y);
    const f2 d01 = fma2(dz01, dz01, fma2(dy01, dy01, mul2(dx01, dx01)));
    const f2 d23 = fma2(dz23, dz23, fma2(dy23, dy23, mul2(dx23, dx23)));
    float u0, u1, u2, u3;
    upk(sub2(cull2, d01), u0, u1);
    upk(sub2(cull2, d23), u2, u3);
    const uint32_t miss = (__float_as_uint(u0) >> 31) | ((__float_as_uint(u1) >> 30) & 2u) |
                          ((__float_as_uint(u2) >> 29) & 4u) | ((__float_as_uint(u3) >> 28) & 8u);
    return miss ^ 0xFu;
}

// ---- per-cell geometry ------------------------------------------------------------------------

struct CellRows {
    uint32_t cbeg, cend;    // the cell's own sorted slots
    uint32_t lo, len, pex;  // lanes 0..8: row r's slot range and its offset in the concatenated list
    uint32_t total;         // candidates in all 9 rows
};

// Row r = (dy, dz) = (r % 3 - 1, r / 3 - 1) of cell c: cells x-1..x+1 of that row, which are
// consecutive keys, hence one slot range [start[first], start[last + 1]).
__device__ __forceinline__ CellRows cell_rows(const uint32_t* __restrict__ start, uint32_t n, int32_t R,
                                              uint32_t R_magic, uint32_t c, uint32_t lane) {
    CellRows cr;
    cr.cend = min(__ldg(start + c + 1), n);
    cr.cbeg = min(__ldg(start + c), cr.cend);
    const uint32_t uR = (uint32_t)R;
    uint32_t rx, ry;
    const uint32_t q = div_R(c, uR, R_magic, &rx);
    const uint32_t qz = div_R(q, uR, R_magic, &ry);
    const int cx = (int)rx, cy = (int)ry, cz = (int)qz;
    uint32_t lo = 0, hi = 0;
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
    cr.lo = lo;
    cr.len = hi - lo;
    uint32_t x = cr.len;
#pragma unroll
    for (int off = 1; off < 16; off <<= 1) {
        const uint32_t y = __shfl_up_sync(FULL, x, off);
        if ((int)lane >= off) x += y;
    }
    cr.pex = x - cr.len;
    cr.total = __shfl_sync(FULL, x, 8);
    return cr;
}

// Split the warp into nt targets x S slices: lane = t + sl * nt. floor() of (a + 0.5) / nt is
// exact here: the fraction is at least 0.5/nt >= 1/64 from an integer and the float error is
// below 1e-5.
struct Team {
    uint32_t S, t, sl;
    bool active;
};
__device__ __forceinline__ Team make_team(uint32_t nt, uint32_t lane) {
    Team tm;
    const float inv = __frcp_rn((float)nt);
    tm.S = (uint32_t)(32.5f * inv);
    tm.sl = (uint32_t)(((float)lane + 0.5f) * inv);
    tm.t = lane - tm.sl * nt;
    tm.active = tm.sl < tm.S;
    return tm;
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

// Staged candidates are tested four at a time: slice sl of a target takes quads sl, sl+S, ...
// (candidates 4q .. 4q+3), so a chunk of targets split S ways runs IT = ceil(ceil(L/4) / S)
// iterations and reads up to 4*S + 8 entries past the list; those entries hold far-away
// positions. Bit strings pack 8 iterations (32 candidates) per 32-bit word; a target's words
// live in its slot hits[ti * MASK_WORDS + w * S + sl] when nwords * S fits the slot.
__device__ __forceinline__ uint32_t stage_padding(uint32_t S) { return 4u * S + 8u; }

struct MaskShape {
    uint32_t IT, nwords;
    bool ok;
};
__device__ __forceinline__ MaskShape mask_shape(uint32_t total, uint32_t S, bool single_chunk) {
    MaskShape ms;
    const uint32_t quads = (total + 3u) >> 2;
    ms.IT = (quads + S - 1u) / S;
    ms.nwords = (ms.IT + 7u) >> 3;
    ms.ok = single_chunk && total + stage_padding(S) <= (uint32_t)STAGE_CAP &&
            ms.nwords * S <= (uint32_t)MASK_WORDS;
    return ms;
}

// Bit strings of a chunk of targets split S ways over L candidates are kept (in any path) when
// every slice's words fit the particle's slot and S <= 8, so that a word's 32 S candidates
// lie within one slot-table piece of the force pass. Both passes decide with this test.
__device__ __forceinline__ bool bits_fit(uint32_t L, uint32_t S) {
    const uint32_t IT = (((L + 3u) >> 2) + S - 1u) / S;
    const uint32_t nwords = (IT + 7u) >> 3;
    return S <= 8u && nwords * S <= (uint32_t)MASK_WORDS;
}

// The split of the last (smallest) chunk of a cell has the most slices, hence the most padding.
__device__ __forceinline__ uint32_t max_slices(uint32_t ncell) {
    const uint32_t rem = ncell & 31u;
    const uint32_t last = rem ? rem : 32u;
    return 32u / last;
}

// slot[j] = the sorted slot of candidate c0 + j of the cell's concatenated list, j < len.
__device__ __forceinline__ void fill_slots(uint32_t* slot, const CellRows& cr, uint32_t c0, uint32_t len,
                                           uint32_t lane) {
    const uint32_t c1 = c0 + len;
#pragma unroll
    for (int r = 0; r < 9; ++r) {
        const uint32_t lo = __shfl_sync(FULL, cr.lo, r);
        const uint32_t rlen = __shfl_sync(FULL, cr.len, r);
        const uint32_t base = __shfl_sync(FULL, cr.pex, r);
        const uint32_t a = max(base, c0), b = min(base + rlen, c1);
        for (uint32_t j = a + lane; j < b; j += 32u) slot[j - c0] = lo + (j - base);
    }
    __syncwarp();
}

// Dense path staging: candidates [c0, c0 + len) of the cell's concatenated list into a CAP-entry
// x/y/z stage (asynchronous copies, one wait), then `pad` far-away entries after them; with
// SLOTS, slot[j] = the sorted slot of staged candidate j. len + pad <= CAP. Callers sync the warp
// before restaging (the previous chunk's readers must be done).
template <int CAP, bool SLOTS>
__device__ __forceinline__ void stage_chunk(float* sx, uint32_t* slot, const CellRows& cr, uint32_t c0, uint32_t len,
                                            uint32_t pad, const float4* __restrict__ pos, uint32_t lane) {
    const uint32_t s0 = (uint32_t)__cvta_generic_to_shared(sx);
    const uint32_t c1 = c0 + len;
#pragma unroll
    for (int r = 0; r < 9; ++r) {
        const uint32_t lo = __shfl_sync(FULL, cr.lo, r);
        const uint32_t rlen = __shfl_sync(FULL, cr.len, r);
        const uint32_t base = __shfl_sync(FULL, cr.pex, r);
        const uint32_t a = max(base, c0), b = min(base + rlen, c1);
        for (uint32_t j = a + lane; j < b; j += 32u) {
            const uint32_t k = lo + (j - base);
            const float* g = reinterpret_cast<const float*>(pos + k);
            const uint32_t at = s0 + 4u * (j - c0);
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(at), "l"(g) : "memory");
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(at + 4u * CAP), "l"(g + 1) : "memory");
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(at + 8u * CAP), "l"(g + 2) : "memory");
            if (SLOTS) slot[j - c0] = k;
        }
    }
    for (uint32_t j = lane; j < pad; j += 32u) {
        sx[len + j] = 1e30f;
        sx[CAP + len + j] = 1e30f;
        sx[2 * CAP + len + j] = 1e30f;
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    __syncwarp();
}

// ---- reference-only terms ---------------------------------------------------------------------

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
        float target = 0.f;
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

// Wall weight functions for a continuous planar wall (WC_FLAG_WALL_WEIGHTS): the density a
// particle at distance d < h gains from one wall, rho0 * 315/256 * P(x) with x = 1 - d/h and
// P(x) = x^5 (16/5 - 16x/3 + 24x^2/7 - x^3 + x^4/9), and the magnitude of the mirrored pressure
// push per unit p rho0 / rho, (30/h) (x^4/4 - x^5/5).
__device__ __forceinline__ float wall_x(float d, float h) { return fminf(fmaxf(1.f - d / h, 0.f), 1.f); }
__device__ __forceinline__ float wall_weight_density(const SceneConsts& c, float x, float y, float z) {
    const float d[6] = {x, c.size - x, y, c.size - y, z, c.size - z};
    float acc = 0.f;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const float s = wall_x(d[k], c.h);
        const float poly = (((s * (1.f / 9.f) - 1.f) * s + 24.f / 7.f) * s - 16.f / 3.f) * s + 16.f / 5.f;
        const float s2 = s * s;
        acc += s2 * s2 * s * poly;
    }
    return c.rho0 * (315.f / 256.f) * acc;
}
__device__ __forceinline__ void wall_weight_push(const SceneConsts& c, const float p[3], float rho, float pressure,
                                                 float f[3]) {
    f[0] = f[1] = f[2] = 0.f;
    if (!(pressure > 0.f)) return;
    const float k = pressure * c.rho0 / rho * (30.f / c.h);
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float lo = wall_x(p[a], c.h), hi = wall_x(c.size - p[a], c.h);
        const float w_lo = lo * lo * lo * lo * (0.25f - 0.2f * lo);
        const float w_hi = hi * hi * hi * hi * (0.25f - 0.2f * hi);
        f[a] = k * (w_lo - w_hi);  // away from the x = 0 wall, away from the x = size wall
    }
}

__device__ __forceinline__ float write_density(const SceneConsts& sc, float sum, uint32_t hits, const float4& pi,
                                               uint32_t ti, float* rho_out, float* p_out, uint32_t* ncount) {
    // The sum includes the particle itself (w = h^2): the reference's m*W(0) term.
    float rho = (sc.m * sc.c6) * sum;
    if (sc.flags & WC_FLAG_WALL_WEIGHTS) rho += wall_weight_density(sc, pi.x, pi.y, pi.z);
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
    if (ncount) ncount[ti] = hits - 1u;
    return total;
}

// The judge step's rates of one particle from its density-pass sums: the Poly6 density rate
// -6 m c6 sum (cull - d2)^2 (r . u) (the time derivative of m c6 sum (cull - d2)^3 with
// d(d2)/dt = 2 r . u), and the pressure rate dp/drho times it for the equation of state. The
// wall terms (wall weights, pseudo wall density) are left out of both.
__device__ __forceinline__ void write_rates(const SceneConsts& sc, float sum, float rr, uint32_t ti,
                                            float2* rate_out) {
    const float rho = (sc.m * sc.c6) * sum;
    const float rate = -6.f * sc.m * sc.c6 * rr;
    float dp;
    if (sc.eos == WC_EOS_LINEAR) {
        dp = sc.k;
    } else {
        const float x = rho / sc.rho0;
        dp = 3.f * sc.k * x * x / sc.rho0;
    }
    rate_out[ti] = make_float2(rate, dp * rate);
}

// Dynamic cell scheduling: every warp takes cells from a counter until it draws an index >= M,
// so a launch of W warps hands out exactly M + W indices and each warp's last draw is one of
// M .. M + W - 1. The warp that draws M + W - 1 draws last; it puts the counter back to zero for
// the next launch (no memset node, and no launch can start from a stale count).
__device__ __forceinline__ void release_counter(uint32_t* counter, uint32_t m_last, uint32_t M, uint32_t lane) {
    if (lane == 0 && m_last == M + gridDim.x * (uint32_t)WARPS - 1u) atomicExch(counter, 0u);
}

// ---- density --------------------------------------------------------------------------------

// BATCHED: cells belong to several scenes (BatchTables); each cell takes its scene's constants
// and indexes the scene's slice of the cell table.
template <bool BATCHED>
__global__ void __launch_bounds__(SPH_THREADS, 5) density_kernel(const SceneConsts sc0, const BatchTables bt,
                                                                 const uint32_t n, const uint32_t num_cells,
                                                                 const float4* __restrict__ pos_in,
                                                                 float* rho_out,  // aliases pos_in[].w
                                                                 float* p_out,    // aliases vel[].w
                                                                 const uint32_t* __restrict__ start,
                                                                 const uint32_t* __restrict__ cell_list,
                                                                 uint32_t* __restrict__ num_nonempty,  // [0] cells, [1]/[2] counters
                                                                 uint32_t* __restrict__ ncount,
                                                                 uint32_t* __restrict__ hits,
                                                                 uint32_t* __restrict__ err) {
    __shared__ __align__(16) float s_stage[WARPS][3][STAGE_CAP];
    __shared__ uint32_t s_coff[BATCHED ? MAX_SCENES + 1 : 1];
    if (BATCHED) {
        for (uint32_t t = threadIdx.x; t <= bt.num_scenes; t += blockDim.x) s_coff[t] = bt.coff[t];
        __syncthreads();
    }
    const uint32_t lane = threadIdx.x & 31u;
    float* sx = s_stage[threadIdx.x >> 5][0];
    float* sy = s_stage[threadIdx.x >> 5][1];
    float* sz = s_stage[threadIdx.x >> 5][2];
    const uint32_t M = min(num_nonempty[0], num_cells);
    // Dynamic scheduling: each warp takes the next cell from a counter (the next index is
    // fetched while the current cell runs), so dense cells do not pile up on a few warps.
    uint32_t* const counter = num_nonempty + 1;
    uint32_t m_next = lane == 0 ? atomicAdd(counter, 1u) : 0u;
    uint32_t m = __shfl_sync(FULL, m_next, 0);
    for (; m < M; m = __shfl_sync(FULL, m_next, 0)) {
        if (lane == 0) m_next = atomicAdd(counter, 1u);
        const uint32_t cg = __ldg(cell_list + m);
        SceneConsts sc;
        uint32_t coff = 0;
        if (BATCHED) {
            const uint32_t s = find_scene(s_coff, bt.num_scenes, cg);
            sc = bt.scenes[s];
            coff = s_coff[s];
        } else {
            sc = sc0;
        }
        const f2 cull2 = pk(sc.cull, sc.cull);
        const CellRows cr = cell_rows(start + coff, n, sc.R, sc.R_magic, cg - coff, lane);
        if (cr.cend - cr.cbeg > MAX_CELL_PARTICLES) {
            // not evaluated (see MAX_CELL_PARTICLES): NaN density and pressure, reported
            for (uint32_t i = cr.cbeg + lane; i < cr.cend; i += 32u) {
                rho_out[4 * (size_t)i] = __int_as_float(0x7fc00000);
                p_out[4 * (size_t)i] = __int_as_float(0x7fc00000);
                if (ncount) ncount[i] = 0u;
            }
            if (lane == 0 && err) atomicOr(err, DEVERR_CELL_OVERFLOW);
            continue;
        }
        const uint32_t pad = stage_padding(max_slices(cr.cend - cr.cbeg));
        if (cr.total + pad <= (uint32_t)STAGE_CAP) {
            // Stage: the concatenated candidate list as x/y/z arrays, then `pad` far-away
            // entries (their d2 overflows to +inf, so they never pass).
            // Asynchronous copies (no registers, all rows in flight at once), one wait.
            const uint32_t s0 = (uint32_t)__cvta_generic_to_shared(sx);
#pragma unroll
            for (int r = 0; r < 9; ++r) {
                const uint32_t lo = __shfl_sync(FULL, cr.lo, r);
                const uint32_t len = __shfl_sync(FULL, cr.len, r);
                const uint32_t base = __shfl_sync(FULL, cr.pex, r);
                for (uint32_t j = lane; j < len; j += 32u) {
                    const float* g = reinterpret_cast<const float*>(pos_in + lo + j);
                    const uint32_t a = s0 + 4u * (base + j);
                    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(a), "l"(g) : "memory");
                    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(a + 4u * STAGE_CAP), "l"(g + 1) : "memory");
                    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(a + 8u * STAGE_CAP), "l"(g + 2) : "memory");
                }
            }
            for (uint32_t j = lane; j < pad; j += 32u) {
                sx[cr.total + j] = 1e30f;
                sy[cr.total + j] = 1e30f;
                sz[cr.total + j] = 1e30f;
            }
            asm volatile("cp.async.wait_all;" ::: "memory");
            __syncwarp();
            const bool single = cr.cend - cr.cbeg <= 32u;
            for (uint32_t t0 = cr.cbeg; t0 < cr.cend; t0 += 32u) {
                const uint32_t nt = min(32u, cr.cend - t0);
                const Team tm = make_team(nt, lane);
                const MaskShape ms = mask_shape(cr.total, tm.S, single);
                const bool store = (ms.ok || bits_fit(cr.total, tm.S)) && hits != nullptr && tm.active;
                const uint32_t ti = t0 + tm.t;
                const float4 pi = pos_in[ti];
                const f2 px = pk(pi.x, pi.x), py = pk(pi.y, pi.y), pz = pk(pi.z, pi.z);
                // Quads are 16-byte aligned (q is a multiple of 4 floats); one 128-bit load gives
                // two packed pairs, the f32x2 operands as they are. y and z follow x in the stage.
                const ulonglong2* qx = reinterpret_cast<const ulonglong2*>(sx) + tm.sl;
                f2 acc01 = 0ull, acc23 = 0ull;  // +0.0f pairs
                uint32_t nh = 0;
                for (uint32_t w = 0; w < ms.nwords; ++w) {
                    uint32_t word = 0;
                    const uint32_t jend = min(8u, ms.IT - 8u * w);
                    if (jend == 8u) {
#pragma unroll
                        for (uint32_t j = 0; j < 8u; ++j, qx += tm.S)
                            word |= quad_hits(qx, px, py, pz, cull2, acc01, acc23) << (4u * j);
                    } else {
#pragma unroll 1
                        for (uint32_t j = 0; j < jend; ++j, qx += tm.S)
                            word |= quad_hits(qx, px, py, pz, cull2, acc01, acc23) << (4u * j);
                    }
                    nh += __popc(word);
                    if (store) hits[(size_t)ti * MASK_WORDS + w * tm.S + tm.sl] = word;
                }
                float a0, a1, a2, a3;
                upk(acc01, a0, a1);
                upk(acc23, a2, a3);
                float sum = (a0 + a1) + (a2 + a3);
                if (!tm.active) {
                    sum = 0.f;
                    nh = 0;
                }
                sum = slice_sum(sum, tm.S, nt, tm.sl);
                nh = slice_sum(nh, tm.S, nt, tm.sl);
                if (tm.sl == 0u) write_density(sc, sum, nh, pi, ti, rho_out, p_out, ncount);
            }
            __syncwarp();  // the stage is rewritten for the next cell
        } else {
            // Dense path (the candidate list does not fit the stage): each chunk of 32 targets
            // streams the list through the stage in pieces and tests it as above. Bit strings
            // are kept when bits_fit: the pieces are then whole words long (32 S candidates a
            // word), so their words form the layout one stage would have given.
            for (uint32_t t0 = cr.cbeg; t0 < cr.cend; t0 += 32u) {
                const uint32_t nt = min(32u, cr.cend - t0);
                const Team tm = make_team(nt, lane);
                const uint32_t ti = t0 + tm.t;
                const float4 pi = pos_in[ti];
                const f2 px = pk(pi.x, pi.x), py = pk(pi.y, pi.y), pz = pk(pi.z, pi.z);
                const uint32_t tpad = stage_padding(tm.S);
                const bool keep = hits != nullptr && bits_fit(cr.total, tm.S);
                const uint32_t room = (uint32_t)STAGE_CAP - tpad;  // a multiple of 4, >= 184
                const uint32_t chunk = keep ? 32u * tm.S * (room / (32u * tm.S)) : room;  // S <= 8: >= 256
                f2 acc01 = 0ull, acc23 = 0ull;
                uint32_t nh = 0, wbase = 0;
                for (uint32_t c0 = 0; c0 < cr.total; c0 += chunk) {
                    const uint32_t len = min(chunk, cr.total - c0);
                    __syncwarp();  // the previous piece's readers are done
                    stage_chunk<STAGE_CAP, false>(sx, nullptr, cr, c0, len, tpad, pos_in, lane);
                    const uint32_t IT = (((len + 3u) >> 2) + tm.S - 1u) / tm.S;
                    const ulonglong2* qx = reinterpret_cast<const ulonglong2*>(sx) + tm.sl;
                    if (keep) {
                        const uint32_t nw = (IT + 7u) >> 3;
                        for (uint32_t w = 0; w < nw; ++w) {
                            uint32_t word = 0;
                            const uint32_t jend = min(8u, IT - 8u * w);
                            if (jend == 8u) {
#pragma unroll
                                for (uint32_t j = 0; j < 8u; ++j, qx += tm.S)
                                    word |= quad_hits(qx, px, py, pz, cull2, acc01, acc23) << (4u * j);
                            } else {
#pragma unroll 1
                                for (uint32_t j = 0; j < jend; ++j, qx += tm.S)
                                    word |= quad_hits(qx, px, py, pz, cull2, acc01, acc23) << (4u * j);
                            }
                            nh += __popc(word);
                            if (tm.active) hits[(size_t)ti * MASK_WORDS + (wbase + w) * tm.S + tm.sl] = word;
                        }
                        wbase += nw;
                    } else {
#pragma unroll 4
                        for (uint32_t j = 0; j < IT; ++j, qx += tm.S)
                            nh += __popc(quad_hits(qx, px, py, pz, cull2, acc01, acc23));
                    }
                }
                float a0, a1, a2, a3;
                upk(acc01, a0, a1);
                upk(acc23, a2, a3);
                float sum = (a0 + a1) + (a2 + a3);
                if (!tm.active) {
                    sum = 0.f;
                    nh = 0;
                }
                sum = slice_sum(sum, tm.S, nt, tm.sl);
                nh = slice_sum(nh, tm.S, nt, tm.sl);
                if (tm.sl == 0u) write_density(sc, sum, nh, pi, ti, rho_out, p_out, ncount);
            }
            __syncwarp();  // the stage is rewritten for the next cell
        }
    }
    release_counter(counter, m, M, lane);
}

// ---- density, one lane per target -------------------------------------------------------------
//
// A warp takes 32 consecutive sorted slots (dynamic scheduling over chunks of 32); each lane owns
// one target, recomputes its cell from its position (the sort's binning) and walks the 9 row
// ranges of the cell's 27 neighbour cells, testing every candidate. Lanes of the same cell walk
// the same candidates in step, so their loads coincide. The target's hits form its bit string in
// its own candidate numbering (bit b of word w: candidate 32 w + b of the rows concatenated),
// kept when it fits the slot (at most 32 MASK_WORDS candidates); the lane force pass reads it.
// FEAT (the learned rollout's judge steps): each hit also adds (cull - d2)^2 (r . u), u = v_i - v_j,
// to the Poly6 density rate (the candidates' velocities from the gather's arrays vxyz, four at a
// time like the positions), and the pass writes rate_out[ti] = (density rate, pressure rate);
// with judge_part it also sums |rho_carried / rho - 1| over each chunk of 32 slots into
// judge_part[m] (rho_carried: the slot's .w before this pass; a non-finite ratio counts 1).

// Rows of the 27 neighbour cells of cell (cx, cy, cz): P[r] = first candidate of row r in the
// concatenated numbering, D[r] = first slot of row r - P[r]; returns the candidate total.
__device__ __forceinline__ uint32_t lane_rows(const uint32_t* __restrict__ tab, uint32_t n, int32_t R, int cx, int cy,
                                              int cz, uint32_t P[9], uint32_t D[9]) {
    uint32_t total = 0;
#pragma unroll
    for (int r = 0; r < 9; ++r) {
        const int yy = cy + (r % 3) - 1, zz = cz + (r / 3) - 1;
        uint32_t lo = 0, hi = 0;
        if (yy >= 0 && yy < R && zz >= 0 && zz < R) {
            const int x0 = cx > 0 ? cx - 1 : 0;
            const int x1 = cx + 1 < R ? cx + 1 : R - 1;
            const uint32_t row = (uint32_t)((zz * R + yy) * R);
            hi = min(__ldg(tab + row + x1 + 1), n);
            lo = min(__ldg(tab + row + x0), hi);
        }
        P[r] = total;
        D[r] = lo - total;
        total += hi - lo;
    }
    return total;
}

template <bool BATCHED, int FEAT = FEAT_NONE>
__global__ void __launch_bounds__(SPH_THREADS, (FEAT == FEAT_FULL && BATCHED) ? 3 : 4) density_lane_kernel(
    const SceneConsts sc0, const BatchTables bt, const uint32_t n, const uint32_t num_cells,
    const float4* pos_in,  // its .w lanes are the density output: read with coherent loads
    float* rho_out, float* p_out, const uint32_t* __restrict__ start, const uint32_t* __restrict__ cell_list,
    uint32_t* __restrict__ num_nonempty,  // [1]: this pass's chunk counter
    uint32_t* __restrict__ ncount, uint32_t* __restrict__ hits, uint32_t* __restrict__ err,
    const float* __restrict__ xyz, const uint32_t xyz_stride,  // the gather's x, y, z arrays
    const float4* vel_in = nullptr,  // FEAT: velocities (their .w lanes are the pressure output)
    const float* __restrict__ vxyz = nullptr, float2* __restrict__ rate_out = nullptr,
    float* __restrict__ judge_part = nullptr) {
    __shared__ uint32_t s_poff[BATCHED ? MAX_SCENES + 1 : 1];
    __shared__ uint32_t s_coff[BATCHED ? MAX_SCENES + 1 : 1];
    if (BATCHED) {
        for (uint32_t t = threadIdx.x; t <= bt.num_scenes; t += blockDim.x) {
            s_poff[t] = bt.poff[t];
            s_coff[t] = bt.coff[t];
        }
        __syncthreads();
    }
    (void)cell_list;
    (void)num_cells;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t M = (n + 31u) >> 5;
    uint32_t* const counter = num_nonempty + 1;
    uint32_t m_next = lane == 0 ? atomicAdd(counter, 1u) : 0u;
    uint32_t m = __shfl_sync(FULL, m_next, 0);
    for (; m < M; m = __shfl_sync(FULL, m_next, 0)) {
        if (lane == 0) m_next = atomicAdd(counter, 1u);
        const uint32_t ti = (m << 5) + lane;
        float judge = 0.f;  // FEAT with judge_part: this slot's |rho_carried / rho - 1|
        do {
        if (ti >= n) break;
        SceneConsts sc;
        uint32_t coff = 0;
        if (BATCHED) {
            const uint32_t s = find_scene(s_poff, bt.num_scenes, ti);
            sc = bt.scenes[s];
            coff = s_coff[s];
        } else {
            sc = sc0;
        }
        const uint32_t* tab = start + coff;
        const float4 pi = pos_in[ti];
        int32_t cx, cy, cz;
        const uint32_t c = bin_key(pi.x, pi.y, pi.z, sc.bin, sc.R, &cx, &cy, &cz);
        const uint32_t cend = min(__ldg(tab + c + 1), n);
        const uint32_t cbeg = min(__ldg(tab + c), cend);
        if (cend - cbeg > MAX_CELL_PARTICLES) {
            // not evaluated (see MAX_CELL_PARTICLES): NaN density and pressure, reported
            rho_out[4 * (size_t)ti] = __int_as_float(0x7fc00000);
            p_out[4 * (size_t)ti] = __int_as_float(0x7fc00000);
            if (ncount) ncount[ti] = 0u;
            if (FEAT == FEAT_FULL) rate_out[ti] = make_float2(0.f, 0.f);
            if (ti == cbeg && err) atomicOr(err, DEVERR_CELL_OVERFLOW);
            judge = 1.f;
            break;
        }
        uint32_t P[9], D[9];
        const uint32_t total = lane_rows(tab, n, sc.R, cx, cy, cz, P, D);
        const bool keep = hits != nullptr && total <= 32u * (uint32_t)MASK_WORDS;
        uint32_t* my_hits = hits ? hits + (size_t)ti * MASK_WORDS : nullptr;
        float4 vi = make_float4(0.f, 0.f, 0.f, 0.f);
        if (FEAT == FEAT_FULL) vi = vel_in[ti];
        float rr = 0.f;  // FEAT: sum of (cull - d2)^2 (r . u)
        const float* X = xyz;
        const float* Y = xyz + xyz_stride;
        const float* Z = xyz + 2 * (size_t)xyz_stride;
        const float* VX = vxyz;
        const float* VY = vxyz + xyz_stride;
        const float* VZ = vxyz + 2 * (size_t)xyz_stride;
        const f2 px = pk(pi.x, pi.x), py = pk(pi.y, pi.y), pz = pk(pi.z, pi.z), cull2 = pk(sc.cull, sc.cull);
        const f2 pvx = pk(vi.x, vi.x), pvy = pk(vi.y, vi.y), pvz = pk(vi.z, vi.z);
        // the weights are added one by one in candidate order, so that the sum does not depend on
        // where the quads fall (a scene of a batch sees the same sums as the scene alone)
        float acc = 0.f;
        uint32_t nh = 0, nbits = 0, wout = 0;
        unsigned long long buf = 0ull;  // hit bits not yet stored, candidate order
#pragma unroll
        for (int r = 0; r < 9; ++r) {
            const uint32_t lo = P[r] + D[r];
            const uint32_t end = lo + ((r < 8 ? P[r + 1] : total) - P[r]);
            // the aligned quads of the x, y, z arrays that cover [lo, end), one 16-byte load per
            // coordinate and the packed f32x2 test (the same fused operations per element as the
            // scalar test); quad places outside the row are masked out
            for (uint32_t k = lo & ~3u; k < end; k += 4u) {
                const ulonglong2 qx = *reinterpret_cast<const ulonglong2*>(X + k);
                const ulonglong2 qy = *reinterpret_cast<const ulonglong2*>(Y + k);
                const ulonglong2 qz = *reinterpret_cast<const ulonglong2*>(Z + k);
                const f2 dx01 = sub2(px, qx.x), dx23 = sub2(px, qx.y);
                const f2 dy01 = sub2(py, qy.x), dy23 = sub2(py, qy.y);
                const f2 dz01 = sub2(pz, qz.x), dz23 = sub2(pz, qz.y);
                const f2 d01 = fma2(dz01, dz01, fma2(dy01, dy01, mul2(dx01, dx01)));
                const f2 d23 = fma2(dz23, dz23, fma2(dy23, dy23, mul2(dx23, dx23)));
                // w = cull - d2 >= 0 exactly when d2 <= cull (the reference's sqrtf(d2) < h; a tie
                // gives +0), and (cull - d2)^3 is Poly6's (h^2 - r^2)^3 with h^2 to the ulp
                float w0, w1, w2, w3;
                upk(sub2(cull2, d01), w0, w1);
                upk(sub2(cull2, d23), w2, w3);
                const uint32_t s0 = lo > k ? lo - k : 0u;
                const uint32_t e0 = min(end - k, 4u);
                const uint32_t valid = (0xFu >> (4u - e0)) & (0xFu << s0);
                const uint32_t miss = (__float_as_uint(w0) >> 31) | ((__float_as_uint(w1) >> 30) & 2u) |
                                      ((__float_as_uint(w2) >> 29) & 4u) | ((__float_as_uint(w3) >> 28) & 8u);
                const uint32_t hit = ~miss & valid;
                const float g0 = (hit & 1u) ? w0 : 0.f, g1 = (hit & 2u) ? w1 : 0.f;
                const float g2 = (hit & 4u) ? w2 : 0.f, g3 = (hit & 8u) ? w3 : 0.f;
                float q0, q1, q2, q3;
                upk(mul2(pk(g0, g1), pk(g0, g1)), q0, q1);
                upk(mul2(pk(g2, g3), pk(g2, g3)), q2, q3);
                acc = fmaf(q0, g0, acc);
                acc = fmaf(q1, g1, acc);
                acc = fmaf(q2, g2, acc);
                acc = fmaf(q3, g3, acc);
                nh += (uint32_t)__popc(hit);
                if (FEAT == FEAT_FULL) {
                    // r . u of the four candidates (packed), added as (cull - d2)^2 (r . u) in order
                    // (loaded for every quad: skipping the quads without hits diverges and was
                    // slower)
                    const ulonglong2 ux = *reinterpret_cast<const ulonglong2*>(VX + k);
                    const ulonglong2 uy = *reinterpret_cast<const ulonglong2*>(VY + k);
                    const ulonglong2 uz = *reinterpret_cast<const ulonglong2*>(VZ + k);
                    const f2 ru01 = fma2(dz01, sub2(pvz, uz.x), fma2(dy01, sub2(pvy, uy.x), mul2(dx01, sub2(pvx, ux.x))));
                    const f2 ru23 = fma2(dz23, sub2(pvz, uz.y), fma2(dy23, sub2(pvy, uy.y), mul2(dx23, sub2(pvx, ux.y))));
                    float r0, r1, r2, r3;
                    upk(ru01, r0, r1);
                    upk(ru23, r2, r3);
                    rr = fmaf(q0, r0, rr);
                    rr = fmaf(q1, r1, rr);
                    rr = fmaf(q2, r2, rr);
                    rr = fmaf(q3, r3, rr);
                }
                buf |= (unsigned long long)(hit >> s0) << nbits;
                nbits += e0 - s0;
                if (nbits >= 32u) {
                    if (keep) my_hits[wout] = (uint32_t)buf;
                    ++wout;
                    buf >>= 32;
                    nbits -= 32u;
                }
            }
        }
        if (keep && nbits) my_hits[wout] = (uint32_t)buf;
        if (FEAT == FEAT_FULL) write_rates(sc, acc, rr, ti, rate_out);
        const float rho_t = write_density(sc, acc, nh, pi, ti, rho_out, p_out, ncount);
        if (FEAT && judge_part) {
            // the ratio in FP32 (relative rounding 1e-7 against a tolerance of order 1e-2)
            const float q = rho_t != 0.f ? fabsf(__fdividef(pi.w, rho_t) - 1.f) : 0.f;
            judge = isfinite(q) ? q : 1.f;
        }
        } while (false);
        if (FEAT && judge_part) {
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) judge += __shfl_xor_sync(FULL, judge, off);
            if (lane == 0) judge_part[m] = judge;
        }
    }
    if (lane == 0 && m == M + gridDim.x * (uint32_t)WARPS - 1u) atomicExch(counter, 0u);
}

// ---- force + integration ------------------------------------------------------------------------

// Accumulators of the force pass per target: NF_PLAIN for the step; FEAT_RATE adds the density
// rate sum, FEAT_FULL the time derivatives of the pair terms.
constexpr int NF_PLAIN = 6, NF_RATE = 7, NF_FEAT = 9;
template <int FEAT>
constexpr int force_accumulators() {
    return FEAT == FEAT_FULL ? NF_FEAT : (FEAT == FEAT_RATE ? NF_RATE : NF_PLAIN);
}

// One neighbour's pressure and viscosity terms. f[0..2] collects pres*(h-d)^2*r/d and f[3..5]
// collects (v_j - v_i)*(h-d)/rho_j; the constant factors are applied once per particle.
// FEAT_FULL (the fast rollout's judge steps): the time derivative of the pressure term, with
// u = v_i - v_j the rate of r, d' = r.u/d the rate of d and the density pass's rates (rho_j',
// p_j' in rj, p_i' in pdot_i): f[6..8] collects
//   (dpres/dt (h-d)^2/d + pres d((h-d)^2/d)/dd d') r + coef u,
//   dpres/dt = (p_i' + p_j') / (2 rho_j) - pres rho_j' / rho_j.
// The viscosity term's derivative is left out: it changes the first-order extrapolation of the
// acceleration by a few percent of its error (1.03 % -> 1.08 % at the first skipped step, FP64
// oracle, 32,768-particle dam break after 300 steps).
// FEAT_RATE (the stale mode's judge steps): f[6] collects the Poly6 density rate sum
// (cull - d2)^2 (r . u) (times -6 m c6 per particle).
template <int FEAT = FEAT_NONE>
__device__ __forceinline__ void pair_terms(const float4& pi, const float4& vi, const float4& pj, const float4& vj,
                                           float h, float cull, float* f, float pdot_i = 0.f,
                                           float2 rj = make_float2(0.f, 0.f)) {
    const float rx = pi.x - pj.x, ry = pi.y - pj.y, rz = pi.z - pj.z;
    const float d2 = dist2(rx, ry, rz);
    const float rsq = d2 > 0.f ? rsqrtf(d2) : 0.f;  // coincident pair (or self): r = 0, no push
    const float d = d2 * rsq;
    const float inv_rho = __fdividef(1.0f, pj.w);
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
    if (FEAT == FEAT_RATE) {
        const float ru = fmaf(rz, vi.z - vj.z, fmaf(ry, vi.y - vj.y, rx * (vi.x - vj.x)));
        const float w = fmaxf(cull - d2, 0.f);
        f[6] = fmaf(w * w, ru, f[6]);
    }
    if (FEAT == FEAT_FULL) {
        const float ux = vi.x - vj.x, uy = vi.y - vj.y, uz = vi.z - vj.z;
        const float ru = fmaf(rz, uz, fmaf(ry, uy, rx * ux));
        const float dp = ru * rsq;  // d'
        if (pres > 0.f) {
            const float g = hd * hd * rsq;
            const float coef = pres * g;
            const float dpres = fmaf(pdot_i + rj.y, 0.5f * inv_rho, -pres * rj.x * inv_rho);
            const float dcoef = -pres * hd * rsq * (2.f + hd * rsq);  // d coef / d d
            const float cr = fmaf(dpres, g, dcoef * dp);
            f[6] = fmaf(cr, rx, fmaf(coef, ux, f[6]));
            f[7] = fmaf(cr, ry, fmaf(coef, uy, f[7]));
            f[8] = fmaf(cr, rz, fmaf(coef, uz, f[8]));
        }
    }
}

// A lane's list (entries list[e * 32 + lane], e < cnt), four entries per round so their loads
// overlap; an empty place takes the particle itself (slot self), whose terms are exactly zero.
// FEAT_FULL: also the neighbours' rates (rate[k]) and the target's pressure rate pdot_i.
template <int FEAT, int ROUND = 4>
__device__ __forceinline__ void accumulate_list(const uint32_t* list, uint32_t cnt, uint32_t lane, uint32_t self,
                                                const float4& pi, const float4& vi, const float4* __restrict__ pos,
                                                const float4* __restrict__ vel, float h, float cull, float* f,
                                                const float2* __restrict__ rate = nullptr, float pdot_i = 0.f) {
    for (uint32_t e = 0; e < cnt; e += (uint32_t)ROUND) {
        uint32_t k[ROUND];
#pragma unroll
        for (int u = 0; u < ROUND; ++u) k[u] = e + (uint32_t)u < cnt ? list[(e + (uint32_t)u) * 32u + lane] : self;
        float4 pj[ROUND], vj[ROUND];
        float2 rj[ROUND];
#pragma unroll
        for (int u = 0; u < ROUND; ++u) {
            pj[u] = __ldg(pos + k[u]);
            vj[u] = __ldg(vel + k[u]);
            rj[u] = FEAT == FEAT_FULL ? __ldg(rate + k[u]) : make_float2(0.f, 0.f);
        }
#pragma unroll
        for (int u = 0; u < ROUND; ++u) pair_terms<FEAT>(pi, vi, pj[u], vj[u], h, cull, f, pdot_i, rj[u]);
    }
}

// Gravity, reference-only external terms, symplectic Euler, speed clamp and wall collision
// (update.comp:145,191-231), then the store into the state buffer.
template <int FEAT>
__device__ __forceinline__ void integrate_store(const SceneConsts& sc, const StepInputs& in, const float4& pi,
                                                const float4& vi, const float* f, uint32_t ti,
                                                float4* __restrict__ pos_a, float4* __restrict__ vel_a,
                                                const uint32_t* __restrict__ ids_b, uint32_t* __restrict__ ids_a,
                                                float4* __restrict__ accel, FeatureBuffers fb = {},
                                                float rate_i = 0.f) {
    const float fp_scale = -sc.m * sc.cs;         // -m * spiky const
    const float fv_scale = sc.m * sc.cv * sc.mu;  // m * visc const * mu
    const float rho = pi.w, pressure = vi.w;
    const float p3[3] = {pi.x, pi.y, pi.z};
    float ext[3] = {in.g[0] * rho, in.g[1] * rho, in.g[2] * rho};
    if (sc.flags & WC_FLAG_WALL_WEIGHTS) {
        float ww[3];
        wall_weight_push(sc, p3, rho, pressure, ww);
#pragma unroll
        for (int a = 0; a < 3; ++a) ext[a] += ww[a];
    }
    if (sc.flags & (WC_FLAG_WALL_FORCE | WC_FLAG_MOUSE_FORCE)) {
        float wf[3] = {0.f, 0.f, 0.f}, mf[3] = {0.f, 0.f, 0.f};
        if (sc.flags & WC_FLAG_WALL_FORCE) wall_forces(sc, p3, wf);
        if (sc.flags & WC_FLAG_MOUSE_FORCE) mouse_force(sc, in, p3, pressure, mf);
#pragma unroll
        for (int a = 0; a < 3; ++a) ext[a] += mf[a] + wf[a];
    }
    const float inv = 1.f / (rho + 1e-16f);
    const float vin[3] = {vi.x, vi.y, vi.z};
    float v[3], x[3], acc[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        // explicit fused operations: the judge steps' variants reuse the products below, and the
        // sum must round the same way in every variant (a judged rollout that reverts every cycle
        // equals plain SPH bit for bit)
        const float force = fmaf(fp_scale, f[a], fmaf(fv_scale, f[3 + a], ext[a]));
        acc[a] = force * inv;
        float va = vin[a] + acc[a] * in.dt;
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
    const float4 pa = make_float4(x[0], x[1], x[2], rho), va = make_float4(v[0], v[1], v[2], pressure);
    pos_a[ti] = pa;
    vel_a[ti] = va;
    if (in.aos_out) {
        in.aos_out[2 * (size_t)ti] = pa;
        in.aos_out[2 * (size_t)ti + 1] = va;
    }
    if (ids_a) ids_a[ti] = ids_b[ti];
    if (accel) accel[ti] = make_float4(acc[0], acc[1], acc[2], 0.f);
    if (FEAT == FEAT_RATE) fb.out[ti] = make_float4(0.f, 0.f, 0.f, -6.f * sc.m * sc.c6 * f[6]);
    if (FEAT == FEAT_FULL) {
        // J = d a / dt of the pressure term: its pair derivatives over rho_i and its share of
        // d(1/rho_i)/dt = -rho_i' / rho_i^2 (the viscosity and external terms' derivatives are
        // left out)
        float jk[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const float pressure_acc = fp_scale * f[a] * inv;
            jk[a] = fmaf(-rate_i * inv, pressure_acc, fp_scale * f[6 + a] * inv);
        }
        fb.out[ti] = make_float4(jk[0], jk[1], jk[2], rate_i);
    }
}

// The learned rollout's judge steps use the lane force pass (force_lane_kernel<.., true>); `fb`
// keeps this kernel's parameters those of the lane kernel (one argument list re-parameterises
// the captured force node of either variant).
template <bool BATCHED>
__global__ void __launch_bounds__(SPH_THREADS, 4) force_kernel(const SceneConsts sc0, const BatchTables bt,
                                                               const StepInputs in, const uint32_t n,
                                                               const uint32_t num_cells,
                                                               const float4* __restrict__ pos_b,
                                                               const float4* __restrict__ vel_b,
                                                               const uint32_t* __restrict__ ids_b,
                                                               float4* __restrict__ pos_a, float4* __restrict__ vel_a,
                                                               uint32_t* __restrict__ ids_a,
                                                               const uint32_t* __restrict__ start,
                                                               const uint32_t* __restrict__ cell_list,
                                                               uint32_t* __restrict__ num_nonempty,  // [0] cells, [1]/[2] counters
                                                               const uint32_t* __restrict__ hits,
                                                               float4* __restrict__ accel,
                                                               uint32_t* __restrict__ err,
                                                               FeatureBuffers fb = {}) {
    (void)fb;
    constexpr int FEAT = FEAT_NONE;
    constexpr int NF = NF_PLAIN;
    // Per warp: the slot table (candidate number -> sorted slot), then the dense path's per-lane
    // lists and its x/y/z stage; the replay path's neighbour lists use both of those regions.
    __shared__ __align__(16) uint32_t s_work[WARPS][STAGE_CAP + FORCE_REPLAY_LIST];
    __shared__ uint32_t s_coff[BATCHED ? MAX_SCENES + 1 : 1];
    if (BATCHED) {
        for (uint32_t t = threadIdx.x; t <= bt.num_scenes; t += blockDim.x) s_coff[t] = bt.coff[t];
        __syncthreads();
    }
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t* slot = s_work[threadIdx.x >> 5];
    uint32_t* list = slot + STAGE_CAP;
    float* fx = reinterpret_cast<float*>(list + FORCE_LIST_CAP * 32);
    const uint32_t M = min(num_nonempty[0], num_cells);
    // Dynamic scheduling: each warp takes the next cell from a counter (the next index is
    // fetched while the current cell runs), so dense cells do not pile up on a few warps.
    uint32_t* const counter = num_nonempty + 2;
    uint32_t m_next = lane == 0 ? atomicAdd(counter, 1u) : 0u;
    uint32_t m = __shfl_sync(FULL, m_next, 0);
    for (; m < M; m = __shfl_sync(FULL, m_next, 0)) {
        if (lane == 0) m_next = atomicAdd(counter, 1u);
        const uint32_t cg = __ldg(cell_list + m);
        SceneConsts sc;
        uint32_t coff = 0;
        if (BATCHED) {
            const uint32_t s = find_scene(s_coff, bt.num_scenes, cg);
            sc = bt.scenes[s];
            coff = s_coff[s];
        } else {
            sc = sc0;
        }
        const CellRows cr = cell_rows(start + coff, n, sc.R, sc.R_magic, cg - coff, lane);
        const uint32_t ncell = cr.cend - cr.cbeg;
        if (ncell > MAX_CELL_PARTICLES) {
            // not evaluated (see MAX_CELL_PARTICLES): the particles keep their state, reported
            for (uint32_t i = cr.cbeg + lane; i < cr.cend; i += 32u) {
                pos_a[i] = pos_b[i];
                vel_a[i] = vel_b[i];
                if (ids_a) ids_a[i] = ids_b[i];
                if (accel) accel[i] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
            if (lane == 0 && err) atomicOr(err, DEVERR_CELL_OVERFLOW);
            continue;
        }
        bool replay = false;
        if (ncell <= 32u && hits != nullptr) {
            const Team tm = make_team(ncell, lane);
            replay = mask_shape(cr.total, tm.S, true).ok;
        }
        if (replay) {
            // Replay the density pass's bit strings: same team, same candidate numbering.
#pragma unroll
            for (int r = 0; r < 9; ++r) {
                const uint32_t lo = __shfl_sync(FULL, cr.lo, r);
                const uint32_t len = __shfl_sync(FULL, cr.len, r);
                const uint32_t base = __shfl_sync(FULL, cr.pex, r);
                for (uint32_t j = lane; j < len; j += 32u) slot[base + j] = lo + j;
            }
            __syncwarp();
            const uint32_t nt = ncell;
            const Team tm = make_team(nt, lane);
            const MaskShape ms = mask_shape(cr.total, tm.S, true);
            const uint32_t ti = cr.cbeg + tm.t;
            const float4 pi = pos_b[ti];
            const float4 vi = vel_b[ti];
            float f[NF] = {};
            // Each lane's hit count, its offset among its target's slices, the target's total,
            // and the target's segment in the warp's neighbour list (targets in order).
            uint32_t cnt = 0;
            if (tm.active)
                for (uint32_t w = 0; w < ms.nwords; ++w) cnt += __popc(__ldg(hits + (size_t)ti * MASK_WORDS + w * tm.S + tm.sl));
            uint32_t inc = cnt;
            for (uint32_t d = 1; d < tm.S; d <<= 1) {
                const uint32_t v = __shfl_up_sync(FULL, inc, d * nt);
                if (tm.sl >= d) inc += v;
            }
            const uint32_t T = __shfl_sync(FULL, inc, tm.t + (tm.S - 1u) * nt);
            const uint32_t tv = lane < nt ? T : 0u;
            uint32_t tinc = tv;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t v = __shfl_up_sync(FULL, tinc, d);
                if ((int)lane >= d) tinc += v;
            }
            const uint32_t all = __shfl_sync(FULL, tinc, 31);
            const uint32_t seg = __shfl_sync(FULL, tinc - tv, tm.t);
            if (all <= (uint32_t)FORCE_REPLAY_LIST) {
                // Decode the bits once into the target's list segment ...
                if (tm.active) {
                    uint32_t at = seg + inc - cnt;
                    const uint32_t s4 = 4u * tm.S;
                    for (uint32_t w = 0; w < ms.nwords; ++w) {
                        uint32_t word = __ldg(hits + (size_t)ti * MASK_WORDS + w * tm.S + tm.sl);
                        const uint32_t qb = 4u * (8u * w * tm.S + tm.sl);
                        while (word) {
                            const uint32_t bit = (uint32_t)__ffs(word) - 1u;
                            word &= word - 1u;
                            const uint32_t q = qb + (bit >> 2) * s4 + (bit & 3u);
                            // Bits always come from this step's density pass over the same
                            // tables; the checks only keep a stage-by-stage caller's stale bits
                            // in bounds (the particle itself contributes exactly zero).
                            uint32_t s = ti;
                            if (q < cr.total) {
                                const uint32_t v = slot[q];
                                if (v < n) s = v;
                            }
                            list[at++] = s;
                        }
                    }
                }
                __syncwarp();
                // ... then the target's slices split its list evenly, four entries per round.
                if (tm.active) {
                    const uint32_t* lst = list + seg;
                    for (uint32_t e = tm.sl; e < T; e += 4u * tm.S) {
                        uint32_t k[4];
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            const uint32_t ee = e + (uint32_t)u * tm.S;
                            k[u] = ee < T ? lst[ee] : ti;
                        }
                        float4 pj[4], vj[4];
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            pj[u] = __ldg(pos_b + k[u]);
                            vj[u] = __ldg(vel_b + k[u]);
                        }
#pragma unroll
                        for (int u = 0; u < 4; ++u) pair_terms<FEAT>(pi, vi, pj[u], vj[u], sc.h, sc.cull, f);
                    }
                }
            } else if (tm.active) {
                for (uint32_t w = 0; w < ms.nwords; ++w) {
                    uint32_t word = __ldg(hits + (size_t)ti * MASK_WORDS + w * tm.S + tm.sl);
                    const uint32_t qb = 4u * (8u * w * tm.S + tm.sl), s4 = 4u * tm.S;
                    while (word) {
                        // Two neighbours per round so their loads overlap; an empty place takes
                        // the particle itself, whose terms are exactly zero.
                        uint32_t k[2];
#pragma unroll
                        for (int u = 0; u < 2; ++u) {
                            k[u] = ti;
                            if (word) {
                                const uint32_t b = (uint32_t)__ffs(word) - 1u;
                                word &= word - 1u;
                                const uint32_t q = qb + (b >> 2) * s4 + (b & 3u);
                                // Bits always come from this step's density pass over the same
                                // tables; the checks only keep a stage-by-stage caller's stale
                                // bits in bounds.
                                if (q < cr.total) {
                                    const uint32_t s = slot[q];
                                    if (s < n) k[u] = s;
                                }
                            }
                        }
                        float4 pj[2], vj[2];
#pragma unroll
                        for (int u = 0; u < 2; ++u) {
                            pj[u] = __ldg(pos_b + k[u]);
                            vj[u] = __ldg(vel_b + k[u]);
                        }
#pragma unroll
                        for (int u = 0; u < 2; ++u) pair_terms<FEAT>(pi, vi, pj[u], vj[u], sc.h, sc.cull, f);
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < NF; ++q) f[q] = slice_sum(f[q], tm.S, nt, tm.sl);
            if (tm.sl == 0u) integrate_store<FEAT>(sc, in, pi, vi, f, ti, pos_a, vel_a, ids_b, ids_a, accel);
            __syncwarp();  // the slot table is rewritten for the next cell
            continue;
        }
        // Chunks of 32 targets. Where the density pass kept bit strings (bits_fit), they are
        // replayed piece by piece: a slot table for the candidates of a few words, each lane
        // decoding its words into its own list, evaluated whenever a list fills. Otherwise the
        // dense path culls: the candidate list streams through the small stage in pieces, the
        // packed test fills the per-lane lists (at most FORCE_DENSE_SLICES slices per target,
        // so a piece keeps most of the stage).
        const f2 cull2 = pk(sc.cull, sc.cull);
        for (uint32_t t0 = cr.cbeg; t0 < cr.cend; t0 += 32u) {
            const uint32_t nt = min(32u, cr.cend - t0);
            Team tm = make_team(nt, lane);
            const uint32_t ti = t0 + tm.t;
            const float4 pi = pos_b[ti];
            const float4 vi = vel_b[ti];
            float f[NF] = {};
            uint32_t cnt = 0;
            if (hits != nullptr && bits_fit(cr.total, tm.S)) {
                const uint32_t IT = (((cr.total + 3u) >> 2) + tm.S - 1u) / tm.S;
                const uint32_t nwords = (IT + 7u) >> 3;
                const uint32_t span = 32u * tm.S;                    // candidates per word
                const uint32_t wpp = (uint32_t)STAGE_CAP / span;      // words per piece, >= 1
                for (uint32_t v0 = 0; v0 < nwords; v0 += wpp) {
                    const uint32_t c0 = v0 * span;
                    const uint32_t len = min(wpp * span, cr.total - c0);
                    __syncwarp();  // the previous piece's readers are done
                    fill_slots(slot, cr, c0, len, lane);
                    const uint32_t v1 = min(v0 + wpp, nwords);
                    for (uint32_t v = v0; v < v1; ++v) {
                        uint32_t word = tm.active ? __ldg(hits + (size_t)ti * MASK_WORDS + v * tm.S + tm.sl) : 0u;
                        const uint32_t qb = 4u * (8u * v * tm.S + tm.sl) - c0;  // first candidate, in the piece
                        for (;;) {
                            while (word && cnt < (uint32_t)REPLAY_LANE_CAP) {
                                const uint32_t b = (uint32_t)__ffs(word) - 1u;
                                word &= word - 1u;
                                const uint32_t q = qb + (b >> 2) * 4u * tm.S + (b & 3u);
                                // Bits always come from this step's density pass over the same
                                // tables; the check only keeps a stage-by-stage caller's stale
                                // bits in bounds (the particle itself contributes exactly zero).
                                list[(cnt++) * 32u + lane] = q < len ? slot[q] : ti;
                            }
                            if (!__any_sync(FULL, word != 0u)) break;
                            accumulate_list<FEAT>(list, cnt, lane, ti, pi, vi, pos_b, vel_b, sc.h, sc.cull, f);
                            cnt = 0;
                        }
                    }
                }
            } else {
                if (tm.S > FORCE_DENSE_SLICES) {
                    tm.S = FORCE_DENSE_SLICES;
                    tm.active = tm.sl < tm.S;
                }
                const f2 px = pk(pi.x, pi.x), py = pk(pi.y, pi.y), pz = pk(pi.z, pi.z);
                const uint32_t tpad = stage_padding(tm.S);
                const uint32_t chunk = (uint32_t)FORCE_STAGE - tpad;  // a multiple of 4, >= 104
                const uint32_t rsl = tm.active ? tm.sl : 0u;          // idle lanes read slice 0, keep nothing
                for (uint32_t c0 = 0; c0 < cr.total; c0 += chunk) {
                    const uint32_t len = min(chunk, cr.total - c0);
                    __syncwarp();  // the previous piece's readers are done
                    stage_chunk<FORCE_STAGE, true>(fx, slot, cr, c0, len, tpad, pos_b, lane);
                    const uint32_t IT = (((len + 3u) >> 2) + tm.S - 1u) / tm.S;
                    const ulonglong2* qx = reinterpret_cast<const ulonglong2*>(fx) + rsl;
                    for (uint32_t j = 0; j < IT; ++j, qx += tm.S) {
                        if (__any_sync(FULL, cnt + 4u > (uint32_t)FORCE_LIST_CAP)) {
                            accumulate_list<FEAT>(list, cnt, lane, ti, pi, vi, pos_b, vel_b, sc.h, sc.cull, f);
                            cnt = 0;
                        }
                        uint32_t bits = quad_test<FORCE_STAGE>(qx, px, py, pz, cull2);
                        if (!tm.active) bits = 0u;
                        const uint32_t qb = 4u * (rsl + j * tm.S);
                        while (bits) {
                            const uint32_t b = (uint32_t)__ffs(bits) - 1u;
                            bits &= bits - 1u;
                            const uint32_t q = qb + b;
                            // The particle itself passes too; it contributes exactly zero. Padding
                            // entries never pass; the check only keeps the read inside the piece.
                            list[(cnt++) * 32u + lane] = q < len ? slot[q] : ti;
                        }
                    }
                }
            }
            accumulate_list<FEAT>(list, cnt, lane, ti, pi, vi, pos_b, vel_b, sc.h, sc.cull, f);
#pragma unroll
            for (int q = 0; q < NF; ++q) f[q] = slice_sum(f[q], tm.S, nt, tm.sl);
            if (tm.sl == 0u) integrate_store<FEAT>(sc, in, pi, vi, f, ti, pos_a, vel_a, ids_b, ids_a, accel);
        }
        __syncwarp();  // the slot table and stage are rewritten for the next cell
    }
    release_counter(counter, m, M, lane);
}

// ---- force + integration, one lane per target ------------------------------------------------
//
// A warp takes 32 consecutive sorted slots (dynamic scheduling over chunks of 32) and each lane
// owns one target. The lane recomputes its cell from its position (the sort's binning) and the 9
// row ranges of the cell's 27 neighbour cells in the density pass's candidate numbering, and
// decodes the target's bit string from the lane density pass (bit b of word w: candidate
// 32 w + b) into a per-lane list of neighbour slots; the list is evaluated four neighbours per
// round whenever it fills. Targets whose bit string was not kept (more than 32 MASK_WORDS
// candidates) test their candidates directly.

constexpr uint32_t LANE_LIST = 48;  // neighbour slots a lane collects before evaluating them (48: 32 and 64 were slower)

// Readback progress (StepInputs part fields): after chunk m every lane fences its stores, and the
// warp that brings its part's count to the part's size publishes the part: the counter goes back
// to zero (no chunk of the part is left in this launch) and, after a system-scope fence, the
// host flag takes this launch's sequence number. No thread waits on anything.
__device__ __forceinline__ void report_chunk(const StepInputs& in, uint32_t m, uint32_t M, uint32_t lane) {
    __threadfence();
    __syncwarp();
    if (lane == 0) {
        const uint32_t r = m / in.part_chunks;
        const uint32_t size = min(in.part_chunks, M - r * in.part_chunks);
        if (atomicAdd(in.part_done + r, 1u) == size - 1u) {
            in.part_done[r] = 0u;
            __threadfence_system();
            *reinterpret_cast<volatile uint32_t*>(in.part_flag + r) = in.seq;
        }
    }
}

// The row of candidate q (the last row whose first candidate is <= q) and its slot, from the row
// starts P[0..8] (P[0] = 0, non-decreasing) and offsets D[r] = first slot of row r - P[r].
__device__ __forceinline__ uint32_t slot_of(uint32_t q, const uint32_t P[9], const uint32_t D[9]) {
    const bool b4 = q >= P[4];
    const bool b2 = q >= (b4 ? P[6] : P[2]);
    const bool b1 = q >= (b4 ? (b2 ? P[7] : P[5]) : (b2 ? P[3] : P[1]));
    uint32_t d = b4 ? (b2 ? (b1 ? D[7] : D[6]) : (b1 ? D[5] : D[4])) : (b2 ? (b1 ? D[3] : D[2]) : (b1 ? D[1] : D[0]));
    if (b4 && b2 && b1 && q >= P[8]) d = D[8];
    return q + d;
}

template <bool BATCHED, int FEAT = FEAT_NONE>
__global__ void __launch_bounds__(SPH_THREADS, (FEAT == FEAT_FULL && BATCHED) ? 2 : 3) force_lane_kernel(
    const SceneConsts sc0, const BatchTables bt, const StepInputs in, const uint32_t n, const uint32_t num_cells,
    const float4* __restrict__ pos_b, const float4* __restrict__ vel_b, const uint32_t* __restrict__ ids_b,
    float4* __restrict__ pos_a, float4* __restrict__ vel_a, uint32_t* __restrict__ ids_a,
    const uint32_t* __restrict__ start, const uint32_t* __restrict__ cell_list,
    uint32_t* __restrict__ num_nonempty,  // [2]: this pass's chunk counter
    const uint32_t* __restrict__ hits, float4* __restrict__ accel, uint32_t* __restrict__ err,
    FeatureBuffers fb = {}) {  // FEAT: the judge step's rates and feature output
    constexpr int NF = force_accumulators<FEAT>();
    __shared__ uint32_t s_list[WARPS][LANE_LIST * 32];
    __shared__ uint32_t s_poff[BATCHED ? MAX_SCENES + 1 : 1];
    __shared__ uint32_t s_coff[BATCHED ? MAX_SCENES + 1 : 1];
    if (BATCHED) {
        for (uint32_t t = threadIdx.x; t <= bt.num_scenes; t += blockDim.x) {
            s_poff[t] = bt.poff[t];
            s_coff[t] = bt.coff[t];
        }
        __syncthreads();
    }
    (void)cell_list;
    (void)num_cells;
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t* list = s_list[threadIdx.x >> 5];
    const uint32_t M = (n + 31u) >> 5;  // chunks of 32 slots
    uint32_t* const counter = num_nonempty + 2;
    uint32_t m_next = lane == 0 ? atomicAdd(counter, 1u) : 0u;
    uint32_t m = __shfl_sync(FULL, m_next, 0);
    for (; m < M; m = __shfl_sync(FULL, m_next, 0)) {
        if (lane == 0) m_next = atomicAdd(counter, 1u);
        const uint32_t ti = (m << 5) + lane;
        const bool live = ti < n;
        const uint32_t tself = live ? ti : n - 1u;
        SceneConsts sc;
        uint32_t coff = 0;
        if (BATCHED) {
            const uint32_t s = find_scene(s_poff, bt.num_scenes, tself);
            sc = bt.scenes[s];
            coff = s_coff[s];
        } else {
            sc = sc0;
        }
        const uint32_t* tab = start + coff;
        const float4 pi = pos_b[tself];
        const float4 vi = vel_b[tself];
        const float2 ri = FEAT == FEAT_FULL ? fb.rate[tself] : make_float2(0.f, 0.f);
        int32_t cx, cy, cz;
        const uint32_t c = bin_key(pi.x, pi.y, pi.z, sc.bin, sc.R, &cx, &cy, &cz);
        const uint32_t cend = min(__ldg(tab + c + 1), n);
        const uint32_t cbeg = min(__ldg(tab + c), cend);
        const uint32_t ncell = cend - cbeg;
        // rows of the 27 neighbour cells, in the density pass's candidate numbering
        uint32_t P[9], D[9];
        const uint32_t total = lane_rows(tab, n, sc.R, cx, cy, cz, P, D);
        const bool overfull = ncell > MAX_CELL_PARTICLES;
        // the lane density pass's bit string: word w, bit b is candidate 32 w + b; kept when the
        // candidates fit the slot
        const uint32_t inchunk = live && !overfull && ti >= cbeg && ti < cend;
        const bool kept = hits != nullptr && total <= 32u * (uint32_t)MASK_WORDS;
        const uint32_t nwords = (total + 31u) >> 5;
        float f[NF] = {};
        // candidate generator state: bit strings (w, word) or direct tests (q)
        bool more = inchunk && total > 0;
        uint32_t w = 0, word = 0, q = 0;
        if (more && kept) word = __ldg(hits + (size_t)ti * MASK_WORDS);
        for (;;) {
            uint32_t cnt = 0;
            while (more && cnt < LANE_LIST) {
                if (kept) {
                    if (word == 0u) {
                        if (++w >= nwords) {
                            more = false;
                            break;
                        }
                        word = __ldg(hits + (size_t)ti * MASK_WORDS + w);
                        continue;
                    }
                    const uint32_t b = (uint32_t)__ffs(word) - 1u;
                    word &= word - 1u;
                    const uint32_t cq = 32u * w + b;
                    // bits always come from this step's density pass over the same tables; the
                    // check only keeps a stage-by-stage caller's stale bits in bounds
                    if (cq < total) {
                        const uint32_t k = slot_of(cq, P, D);
                        list[cnt * 32u + lane] = k < n ? k : ti;
                        ++cnt;
                    }
                } else {
                    if (q >= total) {
                        more = false;
                        break;
                    }
                    const uint32_t k = min(slot_of(q, P, D), n - 1u);
                    ++q;
                    const float4 pj = __ldg(pos_b + k);
                    const float d2 = dist2(pi.x - pj.x, pi.y - pj.y, pi.z - pj.z);
                    if (d2 <= sc.cull) list[(cnt++) * 32u + lane] = k;  // the target itself adds zero
                }
            }
            if (!__any_sync(FULL, cnt > 0u)) break;
            // J (FEAT_FULL) of a single scene: two neighbours per round, so that the pass fits 80
            // registers and three blocks per SM (the batched one keeps four and two blocks)
            accumulate_list<FEAT, (FEAT == FEAT_FULL && !BATCHED) ? 2 : 4>(list, cnt, lane, tself, pi, vi, pos_b, vel_b,
                                                                          sc.h, sc.cull, f, fb.rate, ri.y);
            if (!__any_sync(FULL, more)) break;
        }
        if (live) {
            if (overfull) {
                // not evaluated (see MAX_CELL_PARTICLES): the particle keeps its state, reported
                pos_a[ti] = pi;
                vel_a[ti] = vi;
                if (in.aos_out) {
                    in.aos_out[2 * (size_t)ti] = pi;
                    in.aos_out[2 * (size_t)ti + 1] = vi;
                }
                if (ids_a) ids_a[ti] = ids_b[ti];
                if (accel) accel[ti] = make_float4(0.f, 0.f, 0.f, 0.f);
                if (FEAT) fb.out[ti] = make_float4(0.f, 0.f, 0.f, 0.f);
                if (ti == cbeg && err) atomicOr(err, DEVERR_CELL_OVERFLOW);
            } else {
                integrate_store<FEAT>(sc, in, pi, vi, f, ti, pos_a, vel_a, ids_b, ids_a, accel, fb, ri.x);
            }
        }
        if (in.part_done) report_chunk(in, m, M, lane);
    }
    // the chunk counter returns to zero for the next launch (see release_counter)
    if (lane == 0 && m == M + gridDim.x * (uint32_t)WARPS - 1u) atomicExch(counter, 0u);
}

template <class... A>
constexpr int arity(void (*)(A...)) {
    return (int)sizeof...(A);
}
// A captured step's force node is re-parameterised from ForceKernelArgs: one pointer per
// kernel parameter.
static_assert(arity(&force_kernel<false>) == ForceKernelArgs::COUNT, "ForceKernelArgs out of date");
static_assert(arity(&force_lane_kernel<false, FEAT_NONE>) == ForceKernelArgs::COUNT, "ForceKernelArgs out of date");
static_assert(arity(&force_lane_kernel<true, FEAT_NONE>) == ForceKernelArgs::COUNT, "ForceKernelArgs out of date");

}  // namespace

void sph_occupancy(bool batched, int* density_blocks, int* force_blocks, int pass_variant) {
    int bd = 0, bf = 0;
    if (batched) {
        if (pass_variant == PASSES_LANE)
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bd, density_lane_kernel<true>, SPH_THREADS, 0);
        else
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bd, density_kernel<true>, SPH_THREADS, 0);
        if (pass_variant == PASSES_LANE)
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bf, force_lane_kernel<true>, SPH_THREADS, 0);
        else
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bf, force_kernel<true>, SPH_THREADS, 0);
    } else {
        if (pass_variant == PASSES_LANE)
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bd, density_lane_kernel<false>, SPH_THREADS, 0);
        else
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bd, density_kernel<false>, SPH_THREADS, 0);
        if (pass_variant == PASSES_LANE)
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bf, force_lane_kernel<false>, SPH_THREADS, 0);
        else
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bf, force_kernel<false>, SPH_THREADS, 0);
    }
    *density_blocks = bd > 0 ? bd : 1;
    *force_blocks = bf > 0 ? bf : 1;
}

LaunchDims compute_launch_dims(int device, int pass_variant) {
    LaunchDims ld;
    cudaDeviceGetAttribute(&ld.sms, cudaDevAttrMultiProcessorCount, device);
    if (ld.sms <= 0) ld.sms = 1;
    int bd = 1, bf = 1;
    sph_occupancy(false, &bd, &bf, pass_variant);
    ld.grid_density = ld.sms * bd;
    ld.grid_force = ld.sms * bf;
    ld.grid_stream = ld.sms * 8;
    ld.pass_variant = pass_variant;
    return ld;
}

// The density pass of variant `ld.pass_variant`: its bit strings are laid out for the force pass
// of the same variant.
void launch_density(const DevBuffers& d, const SceneConsts& sc, const LaunchDims& ld, cudaStream_t s) {
    uint32_t* nc = (sc.flags & WC_FLAG_NEIGHBOR_COUNTS) ? d.ncount : nullptr;
    if (ld.pass_variant == PASSES_LANE)
        density_lane_kernel<false><<<ld.grid_density, SPH_THREADS, 0, s>>>(
            sc, BatchTables{}, d.n, d.num_cells, d.pos_b, reinterpret_cast<float*>(d.pos_b) + 3,
            reinterpret_cast<float*>(d.vel_b) + 3, d.start, d.cell_list, d.num_nonempty, nc, d.hits, d.err, d.xyz,
            d.xyz_stride);
    else
        density_kernel<false><<<ld.grid_density, SPH_THREADS, 0, s>>>(
            sc, BatchTables{}, d.n, d.num_cells, d.pos_b, reinterpret_cast<float*>(d.pos_b) + 3,
            reinterpret_cast<float*>(d.vel_b) + 3, d.start, d.cell_list, d.num_nonempty, nc, d.hits, d.err);
}

void launch_density_batched(const DevBuffers& d, const BatchTables& bt, const LaunchDims& ld, cudaStream_t s) {
    if (ld.pass_variant == PASSES_LANE)
        density_lane_kernel<true><<<ld.grid_density, SPH_THREADS, 0, s>>>(
            SceneConsts{}, bt, d.n, d.num_cells, d.pos_b, reinterpret_cast<float*>(d.pos_b) + 3,
            reinterpret_cast<float*>(d.vel_b) + 3, d.start, d.cell_list, d.num_nonempty, d.ncount, d.hits, d.err,
            d.xyz, d.xyz_stride);
    else
        density_kernel<true><<<ld.grid_density, SPH_THREADS, 0, s>>>(
            SceneConsts{}, bt, d.n, d.num_cells, d.pos_b, reinterpret_cast<float*>(d.pos_b) + 3,
            reinterpret_cast<float*>(d.vel_b) + 3, d.start, d.cell_list, d.num_nonempty, d.ncount, d.hits, d.err);
}

// The force pass of variant `ld.pass_variant` on a persistent grid sized from that kernel's
// occupancy; FEAT (the judge steps): the lane kernel with its feature buffers, on a grid of its
// own occupancy.
template <bool BATCHED, int FEAT>
void launch_force_any(const DevBuffers& d, const SceneConsts& sc, const BatchTables& bt, const StepInputs& in,
                      const LaunchDims& ld, FeatureBuffers fb, cudaStream_t s) {
    const bool lane = FEAT != FEAT_NONE || ld.pass_variant == PASSES_LANE;
    int grid = ld.grid_force;
    if (FEAT != FEAT_NONE) {
        static int blocks = 0;
        if (!blocks) {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, force_lane_kernel<BATCHED, FEAT>, SPH_THREADS, 0);
            if (blocks <= 0) blocks = 1;
        }
        grid = ld.sms * blocks;
    }
    if (lane)
        force_lane_kernel<BATCHED, FEAT><<<grid, SPH_THREADS, 0, s>>>(
            sc, bt, in, d.n, d.num_cells, d.pos_b, d.vel_b, d.ids_b, d.pos_a, d.vel_a, d.ids_a, d.start, d.cell_list,
            d.num_nonempty, d.hits, d.accel, d.err, fb);
    else
        force_kernel<BATCHED><<<grid, SPH_THREADS, 0, s>>>(sc, bt, in, d.n, d.num_cells, d.pos_b, d.vel_b, d.ids_b,
                                                          d.pos_a, d.vel_a, d.ids_a, d.start, d.cell_list,
                                                          d.num_nonempty, d.hits, d.accel, d.err, fb);
}

void launch_force(const DevBuffers& d, const SceneConsts& sc, const StepInputs& in, const LaunchDims& ld,
                  cudaStream_t s) {
    launch_force_any<false, FEAT_NONE>(d, sc, BatchTables{}, in, ld, FeatureBuffers{}, s);
}

void launch_force_batched(const DevBuffers& d, const BatchTables& bt, const StepInputs& in, const LaunchDims& ld,
                          cudaStream_t s) {
    launch_force_any<true, FEAT_NONE>(d, SceneConsts{}, bt, in, ld, FeatureBuffers{}, s);
}

void launch_force_feat(const DevBuffers& d, const SceneConsts& sc, const StepInputs& in, const LaunchDims& ld,
                       int level, FeatureBuffers fb, cudaStream_t s) {
    if (level == FEAT_FULL)
        launch_force_any<false, FEAT_FULL>(d, sc, BatchTables{}, in, ld, fb, s);
    else
        launch_force_any<false, FEAT_RATE>(d, sc, BatchTables{}, in, ld, fb, s);
}

void launch_force_batched_feat(const DevBuffers& d, const BatchTables& bt, const StepInputs& in, const LaunchDims& ld,
                               int level, FeatureBuffers fb, cudaStream_t s) {
    if (level == FEAT_FULL)
        launch_force_any<true, FEAT_FULL>(d, SceneConsts{}, bt, in, ld, fb, s);
    else
        launch_force_any<true, FEAT_RATE>(d, SceneConsts{}, bt, in, ld, fb, s);
}

// The judge steps' density pass: the lane kernel with its judge sums (and, FEAT_FULL, rate)
// output, on a grid of its own occupancy, whatever ld.pass_variant says (its bit strings are the
// lane force pass's).
template <bool BATCHED, int FEAT>
void launch_density_any_feat(const DevBuffers& d, const SceneConsts& sc, const BatchTables& bt, const LaunchDims& ld,
                             const float* vxyz, float2* rate, float* judge_part, cudaStream_t s) {
    static int blocks = 0;
    if (!blocks) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, density_lane_kernel<BATCHED, FEAT>, SPH_THREADS, 0);
        if (blocks <= 0) blocks = 1;
    }
    uint32_t* nc = BATCHED ? d.ncount : ((sc.flags & WC_FLAG_NEIGHBOR_COUNTS) ? d.ncount : nullptr);
    density_lane_kernel<BATCHED, FEAT><<<ld.sms * blocks, SPH_THREADS, 0, s>>>(
        sc, bt, d.n, d.num_cells, d.pos_b, reinterpret_cast<float*>(d.pos_b) + 3, reinterpret_cast<float*>(d.vel_b) + 3,
        d.start, d.cell_list, d.num_nonempty, nc, d.hits, d.err, d.xyz, d.xyz_stride, d.vel_b, vxyz, rate, judge_part);
}

void launch_density_feat(const DevBuffers& d, const SceneConsts& sc, const LaunchDims& ld, int level,
                         const float* vxyz, float2* rate, float* judge_part, cudaStream_t s) {
    if (level == FEAT_FULL)
        launch_density_any_feat<false, FEAT_FULL>(d, sc, BatchTables{}, ld, vxyz, rate, judge_part, s);
    else
        launch_density_any_feat<false, FEAT_RATE>(d, sc, BatchTables{}, ld, vxyz, rate, judge_part, s);
}

void launch_density_batched_feat(const DevBuffers& d, const BatchTables& bt, const LaunchDims& ld, int level,
                                 const float* vxyz, float2* rate, float* judge_part, cudaStream_t s) {
    if (level == FEAT_FULL)
        launch_density_any_feat<true, FEAT_FULL>(d, SceneConsts{}, bt, ld, vxyz, rate, judge_part, s);
    else
        launch_density_any_feat<true, FEAT_RATE>(d, SceneConsts{}, bt, ld, vxyz, rate, judge_part, s);
}

const void* force_kernel_symbol(int pass_variant) {
    return pass_variant == PASSES_LANE ? reinterpret_cast<const void*>(&force_lane_kernel<false>)
                                       : reinterpret_cast<const void*>(&force_kernel<false>);
}
const void* force_kernel_batched_symbol(int pass_variant) {
    return pass_variant == PASSES_LANE ? reinterpret_cast<const void*>(&force_lane_kernel<true>)
                                       : reinterpret_cast<const void*>(&force_kernel<true>);
}

}  // namespace wc
