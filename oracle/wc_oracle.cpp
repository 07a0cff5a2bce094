// wc_oracle.cpp — host restatement of WaterCube's particle pipeline. TEST INFRASTRUCTURE ONLY
// (tests, smoke check, CPU-baseline leg of bench.py); the solver never links or calls it.
//
// Built-in semantics (GLSL 4.60 leaves these to the implementation; this file fixes them and the
// GLSL-as-C++ build of the reference shaders in oracle/ref/glsl_compat.h uses the same ones):
//   * length(v) = sqrt(fma(v.z, v.z, fma(v.y, v.y, v.x * v.x)))  (fused; no `precise` in the shaders)
//   * pow(x, y) = powf(x, y)  (C semantics; GLSL leaves x < 0 undefined — this gives sign-correct
//     integer powers, which matters for density.comp:74's z branch that tests p.y)
//   * '/' and sqrt are IEEE round-to-nearest; no other contraction (-ffp-contract=off)
//   * ivec3(float) truncates; NaN -> 0 and out-of-int-range values saturate, then the clamp of
//     count.comp:32 applies (so NaN and -inf bin to cell 0, +inf to cell R-1)
//   * min(x,y) = y < x ? y : x, max(x,y) = x < y ? y : x, clamp = min(max(x,lo),hi)
//   * vec3.length() is the component count 3 (update.comp:77-95 passes it as a distance)
//   * the in-cell order of Sort's atomicAdd ranks (reorder.comp:42) is the input order (stable).
#include "wc_oracle.h"

#include <cmath>
#include <cstring>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---- numeric primitives -----------------------------------------------------------------------

inline float fma_(float a, float b, float c) { return std::fmaf(a, b, c); }
inline double fma_(double a, double b, double c) { return std::fma(a, b, c); }
inline float sqrt_(float a) { return std::sqrt(a); }
inline double sqrt_(double a) { return std::sqrt(a); }
inline float pow_(float a, float b) { return std::pow(a, b); }  // powf
inline double pow_(double a, double b) { return std::pow(a, b); }

template <class T>
inline T gmin(T x, T y) { return y < x ? y : x; }
template <class T>
inline T gmax(T x, T y) { return x < y ? y : x; }
template <class T>
inline T gclamp(T x, T lo, T hi) { return gmin(gmax(x, lo), hi); }

template <class T>
inline T length3(T x, T y, T z) { return sqrt_(fma_(z, z, fma_(y, y, x * x))); }

// ivec3(q) followed by clamp(.., 0, R-1) (count.comp:32).
template <class T>
inline int32_t cell_axis(T q, int32_t R) {
    if (!(q >= T(1))) return 0;           // q < 1 truncates to <= 0; NaN
    if (q >= T(R - 1)) return R - 1;      // trunc(q) >= R-1, incl. +inf
    return (int32_t)q;
}

// ---- constants ------------------------------------------------------------------------------------

template <class T>
struct Consts {
    T size, bin, h, m, rho0, p0, k, mu, c6, cs, cv, max_speed, damping, border;
    T g[3], mo[3], md[3];
    int32_t R;
    uint32_t eos, flags;
};

template <class T>
Consts<T> make_consts(const wc_params& p);

template <>
Consts<float> make_consts<float>(const wc_params& p) {
    Consts<float> c;
    c.size = p.size; c.bin = p.bin_size; c.h = p.kernel_radius; c.m = p.particle_mass;
    c.rho0 = p.rest_density; c.p0 = p.rest_pressure; c.k = p.stiffness; c.mu = p.viscosity;
    c.c6 = p.poly6_const; c.cs = p.spiky_const; c.cv = p.visc_const;
    c.max_speed = p.max_speed; c.damping = p.wall_damping; c.border = p.wall_border;
    for (int a = 0; a < 3; ++a) { c.g[a] = p.gravity[a]; c.mo[a] = p.mouse_origin[a]; c.md[a] = p.mouse_dir[a]; }
    c.R = (int32_t)p.grid_res; c.eos = p.eos; c.flags = p.flags;
    return c;
}

// FP64: the float inputs promoted; the kernel constants evaluated in double from h.
template <>
Consts<double> make_consts<double>(const wc_params& p) {
    Consts<double> c;
    c.size = p.size; c.bin = p.bin_size; c.h = p.kernel_radius; c.m = p.particle_mass;
    c.rho0 = p.rest_density; c.p0 = p.rest_pressure; c.k = p.stiffness; c.mu = p.viscosity;
    const double pi = 3.14159265358979323846;
    c.c6 = 315.0 / (64.0 * pi * std::pow(c.h, 9));
    c.cs = -45.0 / (pi * std::pow(c.h, 6));
    c.cv = 45.0 / (pi * std::pow(c.h, 6));
    c.max_speed = p.max_speed; c.damping = p.wall_damping; c.border = p.wall_border;
    for (int a = 0; a < 3; ++a) { c.g[a] = p.gravity[a]; c.mo[a] = p.mouse_origin[a]; c.md[a] = p.mouse_dir[a]; }
    c.R = (int32_t)p.grid_res; c.eos = p.eos; c.flags = p.flags;
    return c;
}

template <class T>
struct Particle {
    T pos[3];
    T density;
    T vel[3];
    T pressure;
};
static_assert(sizeof(Particle<float>) == sizeof(wc_particle), "layout");
static_assert(sizeof(Particle<double>) == sizeof(wco_particle64), "layout");

template <class T>
inline void cell_of(const Consts<T>& c, const T pos[3], int32_t out[3]) {
    for (int a = 0; a < 3; ++a) out[a] = cell_axis<T>(pos[a] / c.bin, c.R);
}

template <class T>
inline uint32_t key_of(const Consts<T>& c, const int32_t q[3]) {
    return (uint32_t)(q[2] * c.R * c.R + q[1] * c.R + q[0]);
}

// NEIGHBORHOOD of density.comp:40-50 / update.comp:49-59: x outermost, z innermost.
inline void neighbour_offset(int b, int32_t o[3]) {
    o[0] = b / 9 - 1;
    o[1] = (b / 3) % 3 - 1;
    o[2] = b % 3 - 1;
}

// ---- sort: count.comp + linearScan.comp + reorder.comp (+ sort.comp's permutation) -------------

template <class T>
int sort_impl(const wc_params* p, const Particle<T>* in, uint32_t n, Particle<T>* out, uint32_t* keys, uint32_t* perm,
              uint32_t* counts, uint32_t* offsets) {
    const Consts<T> c = make_consts<T>(*p);
    const uint32_t C = (uint32_t)c.R * c.R * c.R;
    std::vector<uint32_t> key(n);
    std::memset(counts, 0, sizeof(uint32_t) * C);  // Sort::clearCountBuffer
    for (uint32_t i = 0; i < n; ++i) {              // count.comp: atomicAdd(counts[index], 1)
        int32_t q[3];
        cell_of(c, in[i].pos, q);
        key[i] = key_of(c, q);
        counts[key[i]] += 1;
    }
    uint32_t prefix = 0;  // linearScan.comp: serial exclusive prefix in key order
    for (uint32_t k = 0; k < C; ++k) {
        offsets[k] = prefix;
        prefix += counts[k];
    }
    std::memset(counts, 0, sizeof(uint32_t) * C);  // clearCountBuffer before reorder
    for (uint32_t i = 0; i < n; ++i) {              // reorder.comp / sort.comp, stable rank
        const uint32_t k = key[i];
        const uint32_t dst = offsets[k] + counts[k]++;
        if (out) out[dst] = in[i];
        if (perm) perm[dst] = i;
    }
    if (keys) std::memcpy(keys, key.data(), sizeof(uint32_t) * n);
    return 0;
}

// ---- density.comp ----------------------------------------------------------------------------

template <class T>
inline T poly6(const Consts<T>& c, T r) {  // density.comp:53-55
    return pow_(c.h * c.h - r * r, T(3)) * c.c6;
}

template <class T>
inline T wall_density(const Consts<T>& c, const T p[3]) {  // density.comp:57-79
    T d = T(0);
    if (p[0] < c.h) d += c.m * poly6(c, p[0]);
    else if (p[0] > c.size - c.h) d += c.m * poly6(c, c.size - p[0]);
    if (p[1] < c.h) d += c.m * poly6(c, p[1]);
    else if (p[1] > c.size - c.h) d += c.m * poly6(c, c.size - p[1]);
    if (p[2] < c.h) d += c.m * poly6(c, p[2]);
    else if (p[1] > c.size - c.h) d += c.m * poly6(c, c.size - p[2]);  // tests p.y, as the shader does
    return d * T(4);
}

// Wall weight functions for a continuous planar wall (WC_FLAG_WALL_WEIGHTS; no counterpart in
// the reference): density rho0 * 315/256 * P(x), x = 1 - d/h, P(x) = x^5 (16/5 - 16x/3 + 24x^2/7
// - x^3 + x^4/9), and the pressure push (p rho0 / rho) (30/h) (x^4/4 - x^5/5) away from the wall.
template <class T>
inline T wall_x(const Consts<T>& c, T d) {
    return gclamp(T(1) - d / c.h, T(0), T(1));
}
template <class T>
inline T wall_weight_density(const Consts<T>& c, const T p[3]) {
    T acc = T(0);
    for (int a = 0; a < 3; ++a) {
        for (int side = 0; side < 2; ++side) {
            const T s = wall_x(c, side ? c.size - p[a] : p[a]);
            const T poly = (((s / T(9) - T(1)) * s + T(24) / T(7)) * s - T(16) / T(3)) * s + T(16) / T(5);
            acc += s * s * s * s * s * poly;
        }
    }
    return c.rho0 * (T(315) / T(256)) * acc;
}
template <class T>
inline void wall_weight_push(const Consts<T>& c, const T p[3], T rho, T pressure, T f[3]) {
    f[0] = f[1] = f[2] = T(0);
    if (!(pressure > T(0))) return;
    const T k = pressure * c.rho0 / rho * (T(30) / c.h);
    for (int a = 0; a < 3; ++a) {
        const T lo = wall_x(c, p[a]), hi = wall_x(c, c.size - p[a]);
        f[a] = k * (lo * lo * lo * lo * (T(0.25) - T(0.2) * lo) - hi * hi * hi * hi * (T(0.25) - T(0.2) * hi));
    }
}

template <class T>
int density_impl(const wc_params* p, Particle<T>* s, uint32_t n, const uint32_t* counts, const uint32_t* offsets,
                 uint32_t* ncount, int threads) {
    const Consts<T> c = make_consts<T>(*p);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256) num_threads(threads > 0 ? threads : omp_get_max_threads())
#endif
    for (int64_t ii = 0; ii < (int64_t)n; ++ii) {
        const uint32_t i = (uint32_t)ii;
        const T* pi = s[i].pos;
        int32_t q[3];
        cell_of(c, pi, q);
        T density = c.m * poly6(c, T(0));
        uint32_t nb = 0;
        for (int b = 0; b < 27; ++b) {
            int32_t o[3];
            neighbour_offset(b, o);
            const int32_t nx = q[0] + o[0], ny = q[1] + o[1], nz = q[2] + o[2];
            if (nx < 0 || ny < 0 || nz < 0 || nx >= c.R || ny >= c.R || nz >= c.R) continue;
            const uint32_t idx = (uint32_t)(nz * c.R * c.R + ny * c.R + nx);
            const uint32_t cnt = counts[idx], off = offsets[idx];
            for (uint32_t l = 0; l < cnt; ++l) {
                const uint32_t j = off + l;
                if (j == i) continue;
                const T* pj = s[j].pos;
                const T dist = length3(pi[0] - pj[0], pi[1] - pj[1], pi[2] - pj[2]);
                if (dist >= c.h) continue;
                density += c.m * poly6(c, dist);
                ++nb;
            }
        }
        if (c.flags & WC_FLAG_WALL_WEIGHTS) density = density + wall_weight_density(c, pi);
        T total = density;
        if (c.flags & WC_FLAG_WALL_DENSITY) total = density + wall_density(c, pi);
        T pressure;
        if (c.eos == WC_EOS_LINEAR)
            pressure = c.p0 + c.k * (density - c.rho0);  // density.comp:129
        else
            pressure = c.p0 + c.k * (pow_(density / c.rho0, T(3)) - T(1));  // density.comp:132-133
        s[i].density = total;
        s[i].pressure = pressure;
        if (ncount) ncount[i] = nb;
    }
    return 0;
}

// ---- update.comp -----------------------------------------------------------------------------

template <class T>
inline void spiky(const Consts<T>& c, const T r[3], T d, T w[3]) {  // update.comp:62-64
    const T s = pow_(c.h - d, T(2));
    for (int a = 0; a < 3; ++a) w[a] = (s * (r[a] / d)) * c.cs;
}

template <class T>
inline void wall_forces(const Consts<T>& c, const T p[3], T f[3]) {  // update.comp:71-100
    f[0] = f[1] = f[2] = T(0);
    const T three = T(3);  // GLSL vec3.length(): the component count
    for (int a = 0; a < 3; ++a) {
        T r[3];
        bool hit = false;
        if (p[a] < c.h) {
            for (int b = 0; b < 3; ++b) r[b] = (b == a ? T(0) : p[b]) - p[b];
            hit = true;
        } else if (p[a] > c.size - c.h) {
            for (int b = 0; b < 3; ++b) r[b] = (b == a ? c.size : p[b]) - p[b];
            hit = true;
        }
        if (hit) {
            T w[3];
            spiky(c, r, three, w);
            for (int b = 0; b < 3; ++b) f[b] += w[b];
        }
    }
    for (int b = 0; b < 3; ++b) f[b] = f[b] * T(0.01);
}

template <class T>
inline void mouse_force(const Consts<T>& c, const Particle<T>& p, T f[3]) {  // update.comp:105-132
    f[0] = f[1] = f[2] = T(0);
    T t1[3], t2[3];
    for (int a = 0; a < 3; ++a) {
        const T tmin = (T(0) - c.mo[a]) / c.md[a];
        const T tmax = (c.size - c.mo[a]) / c.md[a];
        t1[a] = gmin(tmin, tmax);
        t2[a] = gmax(tmin, tmax);
    }
    const T tnear = gmax(gmax(t1[0], t1[1]), t1[2]);
    const T tfar = gmin(gmin(t2[0], t2[1]), t2[2]);
    if (tnear > tfar) return;
    T tm[3];
    for (int a = 0; a < 3; ++a) tm[a] = p.pos[a] - c.mo[a];
    const T* d = c.md;
    const T cx = d[1] * tm[2] - tm[1] * d[2];
    const T cy = d[2] * tm[0] - tm[2] * d[0];
    const T cz = d[0] * tm[1] - tm[0] * d[1];
    const T dist = length3(cx, cy, cz);
    if (dist > c.h) return;
    T w[3];
    spiky(c, tm, dist + T(1e-16), w);
    const T s = -c.m * p.pressure;
    for (int a = 0; a < 3; ++a) f[a] = (s * w[a]) * T(0.00001);
}

template <class T>
int update_impl(const wc_params* p, const Particle<T>* in, Particle<T>* out, uint32_t n, const uint32_t* counts,
                const uint32_t* offsets, T dt, int threads) {
    const Consts<T> c = make_consts<T>(*p);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256) num_threads(threads > 0 ? threads : omp_get_max_threads())
#endif
    for (int64_t ii = 0; ii < (int64_t)n; ++ii) {
        const uint32_t i = (uint32_t)ii;
        const Particle<T>& pi = in[i];
        int32_t q[3];
        cell_of(c, pi.pos, q);
        T pf[3] = {T(0), T(0), T(0)}, vf[3] = {T(0), T(0), T(0)}, ext[3];
        for (int a = 0; a < 3; ++a) ext[a] = c.g[a] * pi.density;
        for (int b = 0; b < 27; ++b) {
            int32_t o[3];
            neighbour_offset(b, o);
            const int32_t nx = q[0] + o[0], ny = q[1] + o[1], nz = q[2] + o[2];
            if (nx < 0 || ny < 0 || nz < 0 || nx >= c.R || ny >= c.R || nz >= c.R) continue;
            const uint32_t idx = (uint32_t)(nz * c.R * c.R + ny * c.R + nx);
            const uint32_t cnt = counts[idx], off = offsets[idx];
            for (uint32_t l = 0; l < cnt; ++l) {
                const uint32_t j = off + l;
                if (j == i) continue;
                const Particle<T>& pj = in[j];
                T r[3];
                for (int a = 0; a < 3; ++a) r[a] = pi.pos[a] - pj.pos[a];
                const T dist = length3(r[0], r[1], r[2]);
                if (dist >= c.h) continue;
                const T pressure = (pi.pressure + pj.pressure) / (T(2) * pj.density);
                if (pressure > T(0)) {
                    T w[3];
                    spiky(c, r, dist + T(1e-16), w);
                    const T s = c.m * pressure;
                    for (int a = 0; a < 3; ++a) pf[a] = pf[a] - s * w[a];
                }
                const T wv = (c.h - dist) * c.cv;
                for (int a = 0; a < 3; ++a) vf[a] = vf[a] + (c.m * ((pj.vel[a] - pi.vel[a]) / pj.density)) * wv;
            }
        }
        if (c.flags & WC_FLAG_WALL_WEIGHTS) {
            T ww[3];
            wall_weight_push(c, pi.pos, pi.density, pi.pressure, ww);
            for (int a = 0; a < 3; ++a) ext[a] = ext[a] + ww[a];
        }
        if (c.flags & (WC_FLAG_MOUSE_FORCE | WC_FLAG_WALL_FORCE)) {
            T mf[3] = {T(0), T(0), T(0)}, wf[3] = {T(0), T(0), T(0)};
            if (c.flags & WC_FLAG_MOUSE_FORCE) mouse_force(c, pi, mf);
            if (c.flags & WC_FLAG_WALL_FORCE) wall_forces(c, pi.pos, wf);
            for (int a = 0; a < 3; ++a) ext[a] = ext[a] + (mf[a] + wf[a]);
        }
        T vel[3], pos[3];
        for (int a = 0; a < 3; ++a) {
            vf[a] = vf[a] * c.mu;
            const T force = (pf[a] + vf[a]) + ext[a];
            const T acc = force / (pi.density + T(1e-16));
            T v = pi.vel[a] + acc * dt;
            if (c.flags & WC_FLAG_SPEED_CLAMP) v = gclamp(v, -c.max_speed, c.max_speed);
            vel[a] = v;
            pos[a] = pi.pos[a] + v * dt;
        }
        for (int a = 0; a < 3; ++a) {  // update.comp:202-227
            if (pos[a] < c.border) {
                vel[a] *= -c.damping;
                pos[a] = c.border;
            } else if (pos[a] > c.size - c.border) {
                vel[a] *= -c.damping;
                pos[a] = c.size - c.border;
            }
        }
        Particle<T>& po = out[i];
        for (int a = 0; a < 3; ++a) { po.pos[a] = pos[a]; po.vel[a] = vel[a]; }
        po.density = pi.density;
        po.pressure = pi.pressure;
    }
    return 0;
}

template <class T>
int step_impl(const wc_params* p, Particle<T>* state, uint32_t n, T dt, uint32_t nsteps, uint32_t* ids, int threads) {
    const uint32_t C = p->grid_res * p->grid_res * p->grid_res;
    std::vector<Particle<T>> sorted(n);
    std::vector<uint32_t> counts(C), offsets(C), perm(n), tmp_ids(ids ? n : 0);
    for (uint32_t s = 0; s < nsteps; ++s) {
        sort_impl<T>(p, state, n, sorted.data(), nullptr, perm.data(), counts.data(), offsets.data());
        if (ids) {
            for (uint32_t k = 0; k < n; ++k) tmp_ids[k] = ids[perm[k]];
            std::memcpy(ids, tmp_ids.data(), sizeof(uint32_t) * n);
        }
        density_impl<T>(p, sorted.data(), n, counts.data(), offsets.data(), nullptr, threads);
        update_impl<T>(p, sorted.data(), state, n, counts.data(), offsets.data(), dt, threads);
    }
    return 0;
}

template <class T>
int diagnostics_impl(const wc_params* p, const Particle<T>* s, uint32_t n, wco_diagnostics* out) {
    const double m = p->particle_mass;
    double mom[3] = {0, 0, 0}, ke = 0, pe = 0;
    for (uint32_t i = 0; i < n; ++i) {
        double v2 = 0, gx = 0;
        for (int a = 0; a < 3; ++a) {
            const double v = (double)s[i].vel[a];
            mom[a] += m * v;
            v2 += v * v;
            gx += (double)p->gravity[a] * (double)s[i].pos[a];
        }
        ke += 0.5 * m * v2;
        pe -= m * gx;
    }
    out->mass = m * n;
    for (int a = 0; a < 3; ++a) out->momentum[a] = mom[a];
    out->kinetic = ke;
    out->potential = pe;
    return 0;
}

inline uint64_t splitmix64(uint64_t& state) {
    uint64_t z = (state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
inline float unit24(uint64_t& state) { return (float)(splitmix64(state) >> 40) * (1.0f / 16777216.0f); }

bool params_ok(const wc_params* p) {
    return p && p->grid_res > 0 && p->grid_res <= 1024 && p->bin_size > 0.0f && p->kernel_radius > 0.0f;
}

}  // namespace

extern "C" {

int wco_sort(const wc_params* p, const wc_particle* in, uint32_t n, wc_particle* out, uint32_t* keys, uint32_t* perm,
             uint32_t* counts, uint32_t* offsets) {
    if (!params_ok(p)) return -1;
    return sort_impl<float>(p, reinterpret_cast<const Particle<float>*>(in), n, reinterpret_cast<Particle<float>*>(out),
                            keys, perm, counts, offsets);
}

int wco_sort64(const wc_params* p, const wco_particle64* in, uint32_t n, wco_particle64* out, uint32_t* keys,
               uint32_t* perm, uint32_t* counts, uint32_t* offsets) {
    if (!params_ok(p)) return -1;
    return sort_impl<double>(p, reinterpret_cast<const Particle<double>*>(in), n,
                             reinterpret_cast<Particle<double>*>(out), keys, perm, counts, offsets);
}

int wco_density_f32(const wc_params* p, wc_particle* sorted, uint32_t n, const uint32_t* counts,
                    const uint32_t* offsets, uint32_t* ncount, int threads) {
    if (!params_ok(p)) return -1;
    return density_impl<float>(p, reinterpret_cast<Particle<float>*>(sorted), n, counts, offsets, ncount, threads);
}

int wco_density_f64(const wc_params* p, wco_particle64* sorted, uint32_t n, const uint32_t* counts,
                    const uint32_t* offsets, uint32_t* ncount, int threads) {
    if (!params_ok(p)) return -1;
    return density_impl<double>(p, reinterpret_cast<Particle<double>*>(sorted), n, counts, offsets, ncount, threads);
}

int wco_update_f32(const wc_params* p, const wc_particle* in, wc_particle* out, uint32_t n, const uint32_t* counts,
                   const uint32_t* offsets, float dt, int threads) {
    if (!params_ok(p)) return -1;
    return update_impl<float>(p, reinterpret_cast<const Particle<float>*>(in), reinterpret_cast<Particle<float>*>(out),
                              n, counts, offsets, dt, threads);
}

int wco_update_f64(const wc_params* p, const wco_particle64* in, wco_particle64* out, uint32_t n,
                   const uint32_t* counts, const uint32_t* offsets, double dt, int threads) {
    if (!params_ok(p)) return -1;
    return update_impl<double>(p, reinterpret_cast<const Particle<double>*>(in),
                               reinterpret_cast<Particle<double>*>(out), n, counts, offsets, dt, threads);
}

int wco_step_f32(const wc_params* p, wc_particle* state, uint32_t n, float dt, uint32_t nsteps, uint32_t* ids,
                 int threads) {
    if (!params_ok(p)) return -1;
    return step_impl<float>(p, reinterpret_cast<Particle<float>*>(state), n, dt, nsteps, ids, threads);
}

int wco_step_f64(const wc_params* p, wco_particle64* state, uint32_t n, double dt, uint32_t nsteps, uint32_t* ids,
                 int threads) {
    if (!params_ok(p)) return -1;
    return step_impl<double>(p, reinterpret_cast<Particle<double>*>(state), n, dt, nsteps, ids, threads);
}

int wco_generate_dam_break(const wc_params* p, uint64_t seed, wc_particle* out, uint32_t n) {
    if (!p || !out) return -1;
    uint32_t a = 1;
    while (2ull * (a + 1) * (a + 1) * (a + 1) <= n) ++a;  // nx = nz = floor(cbrt(n/2))
    const uint32_t nx = a, nz = a;
    const float h = p->kernel_radius;
    const float s = h * 0.5f;
    const float js = 0.01f * h;
    uint64_t st = seed;
    for (uint32_t q = 0; q < n; ++q) {
        const uint32_t i = q % nx, k = (q / nx) % nz, j = q / (nx * nz);
        const float lat[3] = {((float)i + 0.5f) * s, ((float)j + 0.5f) * s, ((float)k + 0.5f) * s};
        wc_particle& o = out[q];
        for (int c = 0; c < 3; ++c) {
            const float u = unit24(st);
            o.position[c] = lat[c] + (2.0f * u - 1.0f) * js;
            o.velocity[c] = 0.0f;
        }
        o.density = 0.0f;
        o.pressure = 0.0f;
    }
    return 0;
}

int wco_generate_reference_lattice(const wc_params* p, uint64_t seed, wc_particle* out, uint32_t n) {
    if (!p || !out) return -1;
    uint32_t d = 1;
    while ((uint64_t)d * d * d < n) ++d;  // ceil(cbrt(n))
    const float distance = p->particle_radius * 1.75f;
    const float jitter = distance * 0.5f;
    uint64_t st = seed;
    for (uint32_t q = 0; q < n; ++q) {
        const uint32_t x = q % d, y = (q / d) % d, z = q / (d * d);
        const float lat[3] = {(float)x * distance, (float)y * distance, (float)z * distance};
        wc_particle& o = out[q];
        for (int c = 0; c < 3; ++c) {
            const float u = unit24(st);
            o.position[c] = lat[c] + (u * jitter - jitter / 2.0f);
            o.velocity[c] = 0.0f;
        }
        o.density = 0.0f;
        o.pressure = 0.0f;
    }
    return 0;
}

// The dam-break workload's constants: h = 0.0457 (16384/n)^(1/3), lattice spacing h/2,
// m = 1000 (h/2)^3, rho0 = 1000, k = 3, mu = 3.5, g = (0, -9.81, 0), linear EOS, restitution 0.5,
// none of the reference-only extras.
int wco_params_dam_break(wc_params* p, uint32_t n) {
    if (!p) return -1;
    std::memset(p, 0, sizeof *p);
    const double h = 0.0457 * std::cbrt(16384.0 / (double)(n ? n : 1));
    const double s = 0.5 * h;
    p->num_particles = n;
    p->size = 1.0f;
    p->kernel_radius = (float)h;
    p->particle_radius = (float)(h / 4.0);
    p->particle_mass = (float)(1000.0 * s * s * s);
    p->rest_density = 1000.0f;
    p->stiffness = 3.0f;
    p->viscosity = 3.5f;
    p->gravity[1] = -9.81f;
    p->time_scale = 1.0f;
    p->eos = WC_EOS_LINEAR;
    p->max_speed = 50.0f;
    p->wall_damping = 0.5f;
    p->wall_border = 0.001f;
    p->mouse_origin[1] = 2.0f;
    p->mouse_dir[1] = 1.0f;
    return 0;
}

// Fluid::setup's derived quantities (src/core/Fluid.cpp:207-216): h = 4 r_p and m = 8 r_p
// when unset, the grid floor(size / h), bin = size / R, and the Poly6 / Spiky / viscosity
// constants evaluated in double and rounded to float, as glm::pow on doubles then the float
// uniform do.
int wco_params_finalize(wc_params* p) {
    if (!p || !(p->size > 0.0f)) return -1;
    if (p->kernel_radius == 0.0f) p->kernel_radius = p->particle_radius * 4.0f;
    if (p->particle_mass == 0.0f) p->particle_mass = p->particle_radius * 8.0f;
    if (!(p->kernel_radius > 0.0f) || !(p->particle_mass > 0.0f)) return -1;
    if (p->grid_res == 0) {
        const float r = std::floor(p->size / p->kernel_radius);
        p->grid_res = r < 1.0f ? 1u : (uint32_t)r;
    }
    if (p->grid_res > 1024) return -1;
    if (p->bin_size == 0.0f) p->bin_size = p->size / (float)p->grid_res;
    const double h = p->kernel_radius;
    const double pi = 3.14159265358979323846;
    if (p->poly6_const == 0.0f) p->poly6_const = (float)(315.0 / (64.0 * pi * std::pow(h, 9)));
    if (p->spiky_const == 0.0f) p->spiky_const = (float)(-45.0 / (pi * std::pow(h, 6)));
    if (p->visc_const == 0.0f) p->visc_const = (float)(45.0 / (pi * std::pow(h, 6)));
    return 0;
}

int wco_diagnostics_f32(const wc_params* p, const wc_particle* s, uint32_t n, wco_diagnostics* out) {
    if (!p || !out) return -1;
    return diagnostics_impl<float>(p, reinterpret_cast<const Particle<float>*>(s), n, out);
}

int wco_diagnostics_f64(const wc_params* p, const wco_particle64* s, uint32_t n, wco_diagnostics* out) {
    if (!p || !out) return -1;
    return diagnostics_impl<double>(p, reinterpret_cast<const Particle<double>*>(s), n, out);
}

float wco_cull_threshold(float h) {
    float x = h * h;
    while (x > 0.0f && !(std::sqrt(x) < h)) x = std::nextafter(x, 0.0f);
    while (std::sqrt(std::nextafter(x, INFINITY)) < h) x = std::nextafter(x, INFINITY);
    return x;
}

int wco_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
