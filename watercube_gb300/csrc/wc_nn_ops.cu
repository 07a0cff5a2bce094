// wc_nn_ops.cu — the surrogate's non-GEMM kernels: radius-h graph from the solver's cell
// tables, node/edge features, LayerNorm forward/backward, ReLU masks, segment sums over the
// receiver-sorted edge list, deterministic column sums, the loss, Adam, weight casts and the
// integrator of a surrogate step. Latent width is 128 throughout (one warp per row, 4 columns
// per lane). All reductions run in a fixed order: results are deterministic.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>

#include "wc_internal.h"
#include "wc_nn.h"

namespace wc {
namespace nn {
namespace {

constexpr unsigned FULL = 0xffffffffu;
constexpr float LN_EPS = 1e-5f;

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
    return v;
}

__device__ __forceinline__ float dist2(float dx, float dy, float dz) {
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

__device__ __forceinline__ int32_t cell_axis(float q, int32_t R) {
    if (!(q >= 1.0f)) return 0;
    if (q >= (float)(R - 1)) return R - 1;
    return (int32_t)q;
}

// ---- graph ------------------------------------------------------------------------------------

// Neighbours of sorted slot i (j != i, |r| < h), visited in increasing slot order: rows of
// increasing key, cells of increasing x. mode 0 counts, mode 1 writes col[].
template <int MODE>
__global__ void graph_kernel(const float4* __restrict__ pos, uint32_t n, const uint32_t* __restrict__ start,
                             float bin, int32_t R, float cull, uint32_t* __restrict__ count,
                             const uint32_t* __restrict__ rowptr, uint32_t* __restrict__ col,
                             uint32_t* __restrict__ err) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = pos[i];
    const int cx = cell_axis(__fdiv_rn(p.x, bin), R), cy = cell_axis(__fdiv_rn(p.y, bin), R),
              cz = cell_axis(__fdiv_rn(p.z, bin), R);
    uint32_t c = 0, w = MODE ? rowptr[i] : 0u;
    for (int dz = -1; dz <= 1; ++dz) {
        const int z = cz + dz;
        if (z < 0 || z >= R) continue;
        for (int dy = -1; dy <= 1; ++dy) {
            const int y = cy + dy;
            if (y < 0 || y >= R) continue;
            const int x0 = cx > 0 ? cx - 1 : 0, x1 = cx + 1 < R ? cx + 1 : R - 1;
            const uint32_t row = (uint32_t)((z * R + y) * R);
            const uint32_t hi = min(start[row + x1 + 1], n), lo = min(start[row + x0], hi);
            if (hi - lo > 3u * MAX_CELL_PARTICLES) {  // a collapsed state: no edges, reported
                if (!MODE) atomicOr(err, DEVERR_CELL_OVERFLOW);
                continue;
            }
            for (uint32_t k = lo; k < hi; ++k) {
                if (k == i) continue;
                const float4 q = __ldg(pos + k);
                if (dist2(p.x - q.x, p.y - q.y, p.z - q.z) <= cull) {
                    if (MODE) col[w++] = k;
                    else ++c;
                }
            }
        }
    }
    if (!MODE) count[i] = c;
}

// recv[e] = receiver of edge e; rev[e] = index of the opposite edge (neighbour lists are
// ascending, so a binary search finds it; the radius graph is symmetric).
__global__ void graph_rev_kernel(uint32_t n, const uint32_t* __restrict__ rowptr, const uint32_t* __restrict__ col,
                                 uint32_t* __restrict__ recv, uint32_t* __restrict__ rev) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (uint32_t e = rowptr[i]; e < rowptr[i + 1]; ++e) {
        const uint32_t j = col[e];
        uint32_t lo = rowptr[j], hi = rowptr[j + 1];
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (col[mid] < i) lo = mid + 1;
            else hi = mid;
        }
        recv[e] = i;
        rev[e] = lo < rowptr[j + 1] && col[lo] == i ? lo : e;  // e only if asymmetric (never for exact tests)
    }
}

// ---- features ---------------------------------------------------------------------------------

// Node features (32, bf16): the last 5 velocities as the current velocity / v_scale (3) and the
// four successive differences (v[s-1] - v[s]) * inv_dv (12; inv_dv = 1 / (dt a_scale), so each is
// a past acceleration on the output scale), wall distances / h clipped to 1 (6), stiffness /
// rest density * 200 (1), the last SPH acceleration / a_scale (3) and its age in steps / 8 (1)
// when one is given (zeros otherwise), zeros (6). hist[s * n + i] is the velocity s steps ago.
// The differences are taken in FP32 before the BF16 cast, which would otherwise lose them.
__global__ void node_features_kernel(uint32_t n, const float4* __restrict__ pos, const float4* __restrict__ hist,
                                     float inv_v, float inv_dv, float inv_h, float size, float k_feature,
                                     const float4* __restrict__ stale, float inv_a, float age_feature,
                                     __nv_bfloat16* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float f[32];
    float4 prev = hist[i];
    f[0] = prev.x * inv_v;
    f[1] = prev.y * inv_v;
    f[2] = prev.z * inv_v;
#pragma unroll
    for (int s = 1; s < 5; ++s) {
        const float4 v = hist[(size_t)s * n + i];
        f[3 * s] = (prev.x - v.x) * inv_dv;
        f[3 * s + 1] = (prev.y - v.y) * inv_dv;
        f[3 * s + 2] = (prev.z - v.z) * inv_dv;
        prev = v;
    }
    const float4 p = pos[i];
    const float w[6] = {p.x, size - p.x, p.y, size - p.y, p.z, size - p.z};
#pragma unroll
    for (int a = 0; a < 6; ++a) f[15 + a] = fminf(fmaxf(w[a] * inv_h, 0.f), 1.f);
    f[21] = k_feature;
#pragma unroll
    for (int a = 22; a < 32; ++a) f[a] = 0.f;
    if (stale) {
        const float4 sa = stale[i];
        f[22] = sa.x * inv_a;
        f[23] = sa.y * inv_a;
        f[24] = sa.z * inv_a;
        f[25] = age_feature;
    }
    __nv_bfloat16* o = out + (size_t)i * 32;
#pragma unroll
    for (int a = 0; a < 32; ++a) o[a] = __float2bfloat16_rn(f[a]);
}

// Edge features (16, bf16): (x_i - x_j) / h (3), |x_i - x_j| / h (1), zeros.
__global__ void edge_features_kernel(uint32_t e_count, const float4* __restrict__ pos, const uint32_t* __restrict__ recv,
                                     const uint32_t* __restrict__ col, float inv_h, __nv_bfloat16* __restrict__ out) {
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= e_count) return;
    const float4 a = pos[recv[e]], b = pos[col[e]];
    const float dx = (a.x - b.x) * inv_h, dy = (a.y - b.y) * inv_h, dz = (a.z - b.z) * inv_h;
    float f[16] = {dx, dy, dz, sqrtf(dx * dx + dy * dy + dz * dz)};
#pragma unroll
    for (int k = 4; k < 16; ++k) f[k] = 0.f;
    __nv_bfloat16* o = out + (size_t)e * 16;
#pragma unroll
    for (int k = 0; k < 16; ++k) o[k] = __float2bfloat16_rn(f[k]);
}

// ---- LayerNorm (width 128) --------------------------------------------------------------------

__global__ void layernorm_kernel(uint32_t rows, const float* __restrict__ y, const float* __restrict__ gamma,
                                 const float* __restrict__ beta, const __nv_bfloat16* __restrict__ resid,
                                 __nv_bfloat16* __restrict__ out, float* __restrict__ mean_out,
                                 float* __restrict__ rstd_out) {
    const uint32_t row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    if (row >= rows) return;
    const float4 v = reinterpret_cast<const float4*>(y + (size_t)row * 128)[lane];
    const float mean = warp_sum(v.x + v.y + v.z + v.w) * (1.f / 128.f);
    const float a = v.x - mean, b = v.y - mean, c = v.z - mean, d = v.w - mean;
    const float var = warp_sum(a * a + b * b + c * c + d * d) * (1.f / 128.f);
    const float rstd = rsqrtf(var + LN_EPS);
    const float4 g = reinterpret_cast<const float4*>(gamma)[lane], bt = reinterpret_cast<const float4*>(beta)[lane];
    float o[4] = {a * rstd * g.x + bt.x, b * rstd * g.y + bt.y, c * rstd * g.z + bt.z, d * rstd * g.w + bt.w};
    if (resid) {
        const __nv_bfloat16* r = resid + (size_t)row * 128 + 4 * lane;
#pragma unroll
        for (int k = 0; k < 4; ++k) o[k] += __bfloat162float(r[k]);
    }
    __nv_bfloat16* dst = out + (size_t)row * 128 + 4 * lane;
#pragma unroll
    for (int k = 0; k < 4; ++k) dst[k] = __float2bfloat16_rn(o[k]);
    if (lane == 0) {
        mean_out[row] = mean;
        rstd_out[row] = rstd;
    }
}

// dy = rstd (g - mean(g) - xhat mean(g xhat)), g = dout * gamma; per-block partial sums of
// dgamma = sum dout xhat and dbeta = sum dout (rows of block b: [b*rpb, (b+1)*rpb)).
constexpr int LNB_WARPS = 8;
__global__ void __launch_bounds__(LNB_WARPS * 32) layernorm_backward_kernel(
    uint32_t rows, uint32_t rows_per_block, const float* __restrict__ dout, const float* __restrict__ y,
    const float* __restrict__ mean, const float* __restrict__ rstd, const float* __restrict__ gamma,
    __nv_bfloat16* __restrict__ dy, float* __restrict__ dy_f32, float* __restrict__ part) {
    __shared__ float s_g[LNB_WARPS][128], s_b[LNB_WARPS][128];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t r0 = blockIdx.x * rows_per_block, r1 = min(rows, r0 + rows_per_block);
    const float4 gm = reinterpret_cast<const float4*>(gamma)[lane];
    float pg[4] = {0.f, 0.f, 0.f, 0.f}, pb[4] = {0.f, 0.f, 0.f, 0.f};
    for (uint32_t row = r0 + warp; row < r1; row += LNB_WARPS) {
        const float4 d = reinterpret_cast<const float4*>(dout + (size_t)row * 128)[lane];
        const float4 v = reinterpret_cast<const float4*>(y + (size_t)row * 128)[lane];
        const float mu = mean[row], rs = rstd[row];
        const float xh[4] = {(v.x - mu) * rs, (v.y - mu) * rs, (v.z - mu) * rs, (v.w - mu) * rs};
        const float dd[4] = {d.x, d.y, d.z, d.w};
        const float gg[4] = {d.x * gm.x, d.y * gm.y, d.z * gm.z, d.w * gm.w};
        const float mg = warp_sum(gg[0] + gg[1] + gg[2] + gg[3]) * (1.f / 128.f);
        const float mgx = warp_sum(gg[0] * xh[0] + gg[1] * xh[1] + gg[2] * xh[2] + gg[3] * xh[3]) * (1.f / 128.f);
        __nv_bfloat16* o = dy + (size_t)row * 128 + 4 * lane;
        float r[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            r[k] = rs * (gg[k] - mg - xh[k] * mgx);
            o[k] = __float2bfloat16_rn(r[k]);
            pg[k] += dd[k] * xh[k];
            pb[k] += dd[k];
        }
        if (dy_f32) *reinterpret_cast<float4*>(dy_f32 + (size_t)row * 128 + 4 * lane) = make_float4(r[0], r[1], r[2], r[3]);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        s_g[warp][4 * lane + k] = pg[k];
        s_b[warp][4 * lane + k] = pb[k];
    }
    __syncthreads();
    if (threadIdx.x < 128) {
        float a = 0.f, b = 0.f;
        for (int w = 0; w < LNB_WARPS; ++w) {
            a += s_g[w][threadIdx.x];
            b += s_b[w][threadIdx.x];
        }
        part[(size_t)blockIdx.x * 256 + threadIdx.x] = a;
        part[(size_t)blockIdx.x * 256 + 128 + threadIdx.x] = b;
    }
}

// ---- elementwise ------------------------------------------------------------------------------

// The ReLU's backward: g = z > 0 ? g : 0, in place (FP32) and as BF16 for the next GEMM.
__global__ void relu_mask_kernel(size_t count, float* __restrict__ g, const __nv_bfloat16* __restrict__ z,
                                 __nv_bfloat16* __restrict__ out) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) {
        const float v = __bfloat162float(z[i]) > 0.f ? g[i] : 0.f;
        g[i] = v;
        out[i] = __float2bfloat16_rn(v);
    }
}

__global__ void cast_kernel(size_t count, const float* __restrict__ x, __nv_bfloat16* __restrict__ out) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
        out[i] = __float2bfloat16_rn(x[i]);
}

// dst[e] += src[idx[e]] (rows of 128).
__global__ void gather_add_kernel(uint32_t rows, const uint32_t* __restrict__ idx, const float* __restrict__ src,
                                  float* __restrict__ dst) {
    const uint32_t row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    if (row >= rows) return;
    const float4 s = reinterpret_cast<const float4*>(src + (size_t)idx[row] * 128)[lane];
    float4* d = reinterpret_cast<float4*>(dst + (size_t)row * 128) + lane;
    float4 v = *d;
    v.x += s.x;
    v.y += s.y;
    v.z += s.z;
    v.w += s.w;
    *d = v;
}

// out[i] = sum over e in [rowptr[i], rowptr[i+1]) of src[idx ? idx[e] : e] (rows of 128).
template <class T>
__global__ void segment_sum_kernel(uint32_t nodes, const uint32_t* __restrict__ rowptr, const uint32_t* __restrict__ idx,
                                   const T* __restrict__ src, float* __restrict__ out_f32,
                                   __nv_bfloat16* __restrict__ out_bf16) {
    const uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    if (i >= nodes) return;
    float a[4] = {0.f, 0.f, 0.f, 0.f};
    for (uint32_t e = rowptr[i]; e < rowptr[i + 1]; ++e) {
        const uint32_t r = idx ? idx[e] : e;
        const T* s = src + (size_t)r * 128 + 4 * lane;
#pragma unroll
        for (int k = 0; k < 4; ++k) a[k] += (float)s[k];
    }
    if (out_f32) {
        *reinterpret_cast<float4*>(out_f32 + (size_t)i * 128 + 4 * lane) = make_float4(a[0], a[1], a[2], a[3]);
    }
    if (out_bf16) {
        __nv_bfloat16* o = out_bf16 + (size_t)i * 128 + 4 * lane;
#pragma unroll
        for (int k = 0; k < 4; ++k) o[k] = __float2bfloat16_rn(a[k]);
    }
}

// part[b][c] = sum of rows [b * rpb, (b+1) * rpb) of column c. Warp w of the block takes rows
// w, w + 8, ...; lane l columns 4l .. 4l+3 (and 128 further per pass); the 8 warps' sums are
// added in a fixed order: deterministic.
constexpr int CS_WARPS = 8;
constexpr uint32_t CS_ROWS = 256;
__global__ void __launch_bounds__(CS_WARPS * 32) colsum_part_kernel(uint32_t rows, uint32_t cols, uint32_t ld,
                                                                   uint32_t rows_per_block, const float* __restrict__ x,
                                                                   float* __restrict__ part) {
    __shared__ float s[CS_WARPS][256];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t r0 = blockIdx.x * rows_per_block, r1 = min(rows, r0 + rows_per_block);
    const bool vec = (cols % 4u == 0) && (ld % 4u == 0) && ((reinterpret_cast<uintptr_t>(x) & 15u) == 0);
    for (uint32_t c0 = 0; c0 < cols; c0 += 128u) {
        float a[4] = {0.f, 0.f, 0.f, 0.f};
        const uint32_t c = c0 + 4u * lane;
        for (uint32_t r = r0 + warp; r < r1; r += CS_WARPS) {
            const float* src = x + (size_t)r * ld + c;
            if (vec) {
                if (c < cols) {
                    const float4 v = *reinterpret_cast<const float4*>(src);
                    a[0] += v.x;
                    a[1] += v.y;
                    a[2] += v.z;
                    a[3] += v.w;
                }
            } else {
#pragma unroll
                for (int k = 0; k < 4; ++k)
                    if (c + k < cols) a[k] += src[k];
            }
        }
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (4u * lane + k < 256u) s[warp][4u * lane + k] = a[k];
        __syncthreads();
        if (threadIdx.x < 128u && c0 + threadIdx.x < cols) {
            float t = 0.f;
            for (int w = 0; w < CS_WARPS; ++w) t += s[w][threadIdx.x];
            part[(size_t)blockIdx.x * cols + c0 + threadIdx.x] = t;
        }
        __syncthreads();
    }
}

// out[c] (+)= sum over blocks of part[b][c], fixed order.
__global__ void colsum_final_kernel(uint32_t blocks, uint32_t cols, const float* __restrict__ part,
                                    float* __restrict__ out, int accumulate) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    float a = 0.f;
    for (uint32_t b = 0; b < blocks; ++b) a += part[(size_t)b * cols + c];
    out[c] = accumulate ? out[c] + a : a;
}

// Mean squared error over 3 components: pred [n x ldp] (normalised), target [n] float4 / scale.
// d_pred = 2 (pred - t) / (3 n) as bf16 (padding columns zero); per-block partial sums of the
// squared error.
__global__ void mse_kernel(uint32_t n, uint32_t ldp, const float* __restrict__ pred, const float4* __restrict__ target,
                           float inv_scale, float* __restrict__ dpred_f32, __nv_bfloat16* __restrict__ dpred,
                           float* __restrict__ part) {
    __shared__ float s[256];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float se = 0.f;
    if (i < n) {
        const float4 t = target[i];
        const float tv[3] = {t.x * inv_scale, t.y * inv_scale, t.z * inv_scale};
        const float g = 2.f / (3.f * (float)n);
        for (uint32_t c = 0; c < ldp; ++c) {
            float d = 0.f;
            if (c < 3) {
                const float diff = pred[(size_t)i * ldp + c] - tv[c];
                se += diff * diff;
                d = g * diff;
            }
            if (dpred) dpred[(size_t)i * ldp + c] = __float2bfloat16_rn(d);
            if (dpred_f32) dpred_f32[(size_t)i * ldp + c] = d;
        }
    }
    s[threadIdx.x] = se;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) s[threadIdx.x] += s[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

// Adam on the FP32 master weights; gradients scaled by grad_scale first.
__global__ void adam_kernel(size_t count, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, float lr, float b1, float b2, float eps, float bc1, float bc2,
                            float grad_scale) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x) {
        const float gi = g[i] * grad_scale;
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    }
}

// W [k_in x n_out] (FP32) -> W^T [n_pad x k_pad] and W [k_pad x n_pad] in BF16, zero padded.
__global__ void cast_weight_kernel(const float* __restrict__ w, uint32_t k_in, uint32_t n_out, uint32_t k_pad,
                                   uint32_t n_pad, __nv_bfloat16* __restrict__ wt, __nv_bfloat16* __restrict__ wk) {
    const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= k_pad * n_pad) return;
    const uint32_t k = idx / n_pad, n = idx % n_pad;
    const float x = (k < k_in && n < n_out) ? w[(size_t)k * n_out + n] : 0.f;
    const __nv_bfloat16 b = __float2bfloat16_rn(x);
    wk[idx] = b;
    wt[(size_t)n * k_pad + k] = b;
}

// A surrogate step: v += a dt (a = network output x a_scale), speed clamp, x += v dt, wall
// collision (the integrator of update.comp:197-227), sorted buffer -> state buffer.
__global__ void integrate_kernel(uint32_t n, const SceneConsts sc, float dt, const float* __restrict__ pred,
                                 uint32_t ldp, float a_scale, const float4* __restrict__ pos_b,
                                 const float4* __restrict__ vel_b, const uint32_t* __restrict__ ids_b,
                                 float4* __restrict__ pos_a, float4* __restrict__ vel_a, uint32_t* __restrict__ ids_a) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = pos_b[i], v = vel_b[i];
    const float pp[3] = {p.x, p.y, p.z}, vv[3] = {v.x, v.y, v.z};
    float x[3], u[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        float va = vv[a] + pred[(size_t)i * ldp + a] * a_scale * dt;
        if (sc.flags & WC_FLAG_SPEED_CLAMP) va = fminf(fmaxf(va, -sc.max_speed), sc.max_speed);
        float xa = pp[a] + va * dt;
        if (xa < sc.border) {
            va *= -sc.damping;
            xa = sc.border;
        } else if (xa > sc.size - sc.border) {
            va *= -sc.damping;
            xa = sc.size - sc.border;
        }
        x[a] = xa;
        u[a] = va;
    }
    pos_a[i] = make_float4(x[0], x[1], x[2], p.w);
    vel_a[i] = make_float4(u[0], u[1], u[2], v.w);
    if (ids_a) ids_a[i] = ids_b[i];
}

// out[perm[k]] style gather of float4 rows: dst[k] = src[perm[k]] (history follows the sort).
// dst.xyz -= sub.xyz (the target of a residual sample: the change since the stale acceleration)
__global__ void sub_xyz_kernel(uint32_t n, float4* __restrict__ dst, const float4* __restrict__ sub) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 a = dst[i];
    const float4 b = sub[i];
    a.x -= b.x;
    a.y -= b.y;
    a.z -= b.z;
    dst[i] = a;
}

// dst = base + scale * pred[:, 0:3] (a residual prediction added to the stale acceleration)
__global__ void add_scaled_kernel(uint32_t n, const float* __restrict__ pred, uint32_t ldp, float scale,
                                  const float4* __restrict__ base, float4* __restrict__ dst) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* p = pred + (size_t)i * ldp;
    const float4 b = base[i];
    dst[i] = make_float4(__fmaf_rn(p[0], scale, b.x), __fmaf_rn(p[1], scale, b.y), __fmaf_rn(p[2], scale, b.z), 0.f);
}

__global__ void gather4_kernel(uint32_t n, const uint32_t* __restrict__ perm, const float4* __restrict__ src,
                               float4* __restrict__ dst) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = src[perm[i]];
}

// dst[ids[k]] = src[k].w (per-id density), for density comparisons across two orders.
__global__ void scatter_density_kernel(uint32_t n, const uint32_t* __restrict__ ids, const float4* __restrict__ src,
                                       float* __restrict__ dst) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[ids[i]] = src[i].w;
}

// part[b] = sum over the block's i of |a[i] / b[i] - 1| (FP64).
__global__ void rel_err_kernel(uint32_t n, const float* __restrict__ a, const float* __restrict__ b,
                               double* __restrict__ part) {
    __shared__ double s[256];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    s[threadIdx.x] = i < n ? fabs((double)a[i] / (double)b[i] - 1.0) : 0.0;
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) s[threadIdx.x] += s[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

inline unsigned blocks_for(size_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

void graph_count(const float4* pos, uint32_t n, const uint32_t* start, float bin, int32_t R, float cull,
                 uint32_t* count, uint32_t* err, cudaStream_t s) {
    if (n) graph_kernel<0><<<blocks_for(n, 128), 128, 0, s>>>(pos, n, start, bin, R, cull, count, nullptr, nullptr, err);
}
void graph_fill(const float4* pos, uint32_t n, const uint32_t* start, float bin, int32_t R, float cull,
                const uint32_t* rowptr, uint32_t* col, cudaStream_t s) {
    if (n) graph_kernel<1><<<blocks_for(n, 128), 128, 0, s>>>(pos, n, start, bin, R, cull, nullptr, rowptr, col, nullptr);
}
void graph_rev(uint32_t n, const uint32_t* rowptr, const uint32_t* col, uint32_t* recv, uint32_t* rev, cudaStream_t s) {
    if (n) graph_rev_kernel<<<blocks_for(n, 128), 128, 0, s>>>(n, rowptr, col, recv, rev);
}
void node_features(uint32_t n, const float4* pos, const float4* hist, float inv_v, float inv_dv, float inv_h,
                   float size, float k_feature, const float4* stale, float inv_a, float age_feature,
                   __nv_bfloat16* out, cudaStream_t s) {
    if (n)
        node_features_kernel<<<blocks_for(n, 128), 128, 0, s>>>(n, pos, hist, inv_v, inv_dv, inv_h, size, k_feature,
                                                                stale, inv_a, age_feature, out);
}
void edge_features(uint32_t e, const float4* pos, const uint32_t* recv, const uint32_t* col, float inv_h,
                   __nv_bfloat16* out, cudaStream_t s) {
    if (e) edge_features_kernel<<<blocks_for(e, 256), 256, 0, s>>>(e, pos, recv, col, inv_h, out);
}
void layernorm(uint32_t rows, const float* y, const float* gamma, const float* beta, const __nv_bfloat16* resid,
               __nv_bfloat16* out, float* mean, float* rstd, cudaStream_t s) {
    if (rows) layernorm_kernel<<<blocks_for((size_t)rows * 32, 256), 256, 0, s>>>(rows, y, gamma, beta, resid, out, mean, rstd);
}
uint32_t layernorm_backward_blocks(uint32_t rows) { return rows ? blocks_for(rows, 512) : 0; }
void layernorm_backward(uint32_t rows, const float* dout, const float* y, const float* mean, const float* rstd,
                        const float* gamma, __nv_bfloat16* dy, float* dy_f32, float* part, cudaStream_t s) {
    const uint32_t blocks = layernorm_backward_blocks(rows);
    if (blocks)
        layernorm_backward_kernel<<<blocks, LNB_WARPS * 32, 0, s>>>(rows, 512, dout, y, mean, rstd, gamma, dy, dy_f32,
                                                                    part);
}
void relu_mask(size_t count, float* g, const __nv_bfloat16* z, __nv_bfloat16* out, cudaStream_t s) {
    if (count) relu_mask_kernel<<<(unsigned)std::min<size_t>(blocks_for(count, 256), 65535), 256, 0, s>>>(count, g, z, out);
}
void cast_bf16(size_t count, const float* x, __nv_bfloat16* out, cudaStream_t s) {
    if (count) cast_kernel<<<(unsigned)std::min<size_t>(blocks_for(count, 256), 65535), 256, 0, s>>>(count, x, out);
}
void gather_add(uint32_t rows, const uint32_t* idx, const float* src, float* dst, cudaStream_t s) {
    if (rows) gather_add_kernel<<<blocks_for((size_t)rows * 32, 256), 256, 0, s>>>(rows, idx, src, dst);
}
void segment_sum_bf16(uint32_t nodes, const uint32_t* rowptr, const uint32_t* idx, const __nv_bfloat16* src,
                      float* out_f32, __nv_bfloat16* out_bf16, cudaStream_t s) {
    if (nodes)
        segment_sum_kernel<__nv_bfloat16><<<blocks_for((size_t)nodes * 32, 256), 256, 0, s>>>(nodes, rowptr, idx, src,
                                                                                             out_f32, out_bf16);
}
void segment_sum_f32(uint32_t nodes, const uint32_t* rowptr, const uint32_t* idx, const float* src, float* out_f32,
                     __nv_bfloat16* out_bf16, cudaStream_t s) {
    if (nodes)
        segment_sum_kernel<float><<<blocks_for((size_t)nodes * 32, 256), 256, 0, s>>>(nodes, rowptr, idx, src, out_f32,
                                                                                     out_bf16);
}
uint32_t colsum_blocks(uint32_t rows) { return rows ? blocks_for(rows, CS_ROWS) : 0; }
void colsum(uint32_t rows, uint32_t cols, uint32_t ld, const float* x, float* part, float* out, int accumulate,
            cudaStream_t s) {
    const uint32_t blocks = colsum_blocks(rows);
    if (!blocks) return;
    colsum_part_kernel<<<blocks, CS_WARPS * 32, 0, s>>>(rows, cols, ld, CS_ROWS, x, part);
    colsum_final_kernel<<<blocks_for(cols, 128), 128, 0, s>>>(blocks, cols, part, out, accumulate);
}
void colsum_partials(uint32_t blocks, uint32_t cols, const float* part, float* out, int accumulate, cudaStream_t s) {
    if (blocks) colsum_final_kernel<<<blocks_for(cols, 128), 128, 0, s>>>(blocks, cols, part, out, accumulate);
}
uint32_t mse_blocks(uint32_t n) { return n ? blocks_for(n, 256) : 0; }
void mse(uint32_t n, uint32_t ldp, const float* pred, const float4* target, float inv_scale, float* dpred_f32,
         __nv_bfloat16* dpred, float* part, cudaStream_t s) {
    if (n) mse_kernel<<<mse_blocks(n), 256, 0, s>>>(n, ldp, pred, target, inv_scale, dpred_f32, dpred, part);
}
void adam(size_t count, float* w, const float* g, float* m, float* v, float lr, float b1, float b2, float eps,
          int step, float grad_scale, cudaStream_t s) {
    const float bc1 = 1.f - powf(b1, (float)step), bc2 = 1.f - powf(b2, (float)step);
    if (count)
        adam_kernel<<<(unsigned)std::min<size_t>(blocks_for(count, 256), 4096), 256, 0, s>>>(count, w, g, m, v, lr, b1, b2,
                                                                                      eps, bc1, bc2, grad_scale);
}
void cast_weight(const float* w, uint32_t k_in, uint32_t n_out, uint32_t k_pad, uint32_t n_pad, __nv_bfloat16* wt,
                 __nv_bfloat16* wk, cudaStream_t s) {
    cast_weight_kernel<<<blocks_for((size_t)k_pad * n_pad, 256), 256, 0, s>>>(w, k_in, n_out, k_pad, n_pad, wt, wk);
}
void integrate(uint32_t n, const SceneConsts& sc, float dt, const float* pred, uint32_t ldp, float a_scale,
               const DevBuffers& d, cudaStream_t s) {
    if (n)
        integrate_kernel<<<blocks_for(n, 256), 256, 0, s>>>(n, sc, dt, pred, ldp, a_scale, d.pos_b, d.vel_b, d.ids_b,
                                                            d.pos_a, d.vel_a, d.ids_a);
}
void sub_xyz(uint32_t n, float4* dst, const float4* sub, cudaStream_t s) {
    if (n) sub_xyz_kernel<<<blocks_for(n, 256), 256, 0, s>>>(n, dst, sub);
}
void add_scaled(uint32_t n, const float* pred, uint32_t ldp, float scale, const float4* base, float4* dst,
                cudaStream_t s) {
    if (n) add_scaled_kernel<<<blocks_for(n, 256), 256, 0, s>>>(n, pred, ldp, scale, base, dst);
}
void gather4(uint32_t n, const uint32_t* perm, const float4* src, float4* dst, cudaStream_t s) {
    if (n) gather4_kernel<<<blocks_for(n, 256), 256, 0, s>>>(n, perm, src, dst);
}
void scatter_density(uint32_t n, const uint32_t* ids, const float4* src, float* dst, cudaStream_t s) {
    if (n) scatter_density_kernel<<<blocks_for(n, 256), 256, 0, s>>>(n, ids, src, dst);
}
uint32_t rel_err_blocks(uint32_t n) { return n ? blocks_for(n, 256) : 0; }
void rel_err(uint32_t n, const float* a, const float* b, double* part, cudaStream_t s) {
    if (n) rel_err_kernel<<<rel_err_blocks(n), 256, 0, s>>>(n, a, b, part);
}

}  // namespace nn
}  // namespace wc
