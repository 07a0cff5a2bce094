// wc_local.cu — the fast rollout (no counterpart in the reference).
//
// Every K-th step is a plain SPH step, the judge. Its density pass also computes each
// particle's density and pressure rates (density_lane_kernel<.., FEAT>), and its force pass the
// time derivative J of the SPH acceleration with the neighbours' rates (force_lane_kernel<..,
// FEAT>). The K - 1 steps after it run without neighbour passes on
//
//   a(t + k) = a(t)                          WC_LOCAL_STALE
//   a(t + k) = a(t) + k dt J                 WC_LOCAL_TAYLOR
//   a(t + k) = a(t) + k dt J + a_s r_k       WC_LOCAL_NETWORK
//
// where r_k is a per-particle network's residual of the Taylor term, from 19 inputs of the judge
// step (with its mean over the particles removed):
//
//   x  = [a / a_s, J T / a_s, 100 rhodot T / rho, v / v_s, rho / rho0 - 1, p / (k rho0),
//         six wall distances / h (clipped to [0, 1]), 100 k / rho0]            (19, padded to 32)
//   h1 = relu(W1 x + b1) (64),  h2 = relu(W2 h1 + b2) (64),  r = W3 h2 + b3 (16, 3 ages used each)
//
// with the network's time unit T = DT_REF = 1 ms; r is in units of a_s (dt / T)^2, the way the
// residual of a first-order extrapolation scales with the time step, so that the network serves
// every dt.
//
// Inference is one kernel per judge step (mlp_kernel): per 128-particle tile the inputs are
// computed into shared memory in the tensor cores' K-major core-matrix layout, and the three
// layers run as tcgen05.mma (BF16 x BF16 -> FP32 in tensor memory), each epilogue reading the
// accumulator with tcgen05.ld, adding the bias, applying ReLU and writing the next layer's BF16
// operand back to shared memory. The skipped steps integrate in one kernel and carry each
// particle's density by its rate; the next judge step compares that carried density with the
// SPH density of the same particles and reverts the cycle when the mean
// |rho_carried / rho_SPH - 1| exceeds the tolerance.
//
// Training (wc_local_record_*, wc_local_train) runs on trajectories of the solver itself:
// samples are the judge step's inputs and the residuals (a(t + k) - a(t) - k dt J) / a_s of the
// SPH accelerations of the next `ages` steps, matched by particle id; the network is trained by
// Adam with the tcgen05 GEMM of wc_nn_gemm.cu for the forward and the hand-written backward pass.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "wc_internal.h"
#include "wc_nn.h"
#include "wc_util.h"

using namespace wc;

namespace {

constexpr uint32_t IN = 32, IN_USED = 19, HID = 64, OUT = 16, MAX_AGES = 5;
// A sample's targets: YW floats, the residuals of ages 1 .. MAX_AGES in columns 0 .. 3 MAX_AGES - 1,
// then (DT_REF / dt)^2 in column RES_SCALE and dt J / a_s in columns JD .. JD + 2.
constexpr uint32_t YW = 20, RES_SCALE = 16, JD = 17;
// The network's changes per particle in a rollout: 3 MAX_AGES columns padded to 16 (whole 16-byte stores).
constexpr uint32_t CHANGE_LD = 16;
static_assert(3 * MAX_AGES <= OUT && 3 * MAX_AGES <= RES_SCALE && 3 * MAX_AGES <= CHANGE_LD, "ages do not fit");
constexpr uint32_t TILE = 128;
constexpr uint32_t MLP_THREADS = 128;
constexpr uint32_t MLP_CTAS_PER_SM = 6;
constexpr uint32_t TMEM_COLS = 64;
static_assert(MLP_THREADS == TILE && TILE == 128 && OUT == 16, "mlp_kernel: one thread per row, 4 warps, 16 outputs");
constexpr uint32_t WAIT_LIMIT = 1u << 22;
// The network's time unit: its J and density-rate inputs are J DT_REF / a_s and
// 100 rhodot DT_REF / rho, and it learns the residual of the Taylor term in units of
// a_s (dt / DT_REF)^2 (the residual grows with the square of the time step), so that one network
// serves every dt. Column RES_SCALE of a sample's targets holds (DT_REF / dt)^2.
constexpr float DT_REF = 1e-3f;

// FP32 master parameters, W as [k_in x n_out] row-major (the convention of cast_weight).
constexpr size_t OFF_W1 = 0;
constexpr size_t OFF_B1 = OFF_W1 + (size_t)IN * HID;
constexpr size_t OFF_W2 = OFF_B1 + HID;
constexpr size_t OFF_B2 = OFF_W2 + (size_t)HID * HID;
constexpr size_t OFF_W3 = OFF_B2 + HID;
constexpr size_t OFF_B3 = OFF_W3 + (size_t)HID * OUT;
constexpr size_t NPARAMS = OFF_B3 + OUT;
// BF16 copies: W^T [n_out x k_in] (forward operand) and W [k_in x n_out] (input-gradient operand).
constexpr size_t BF_W1T = 0, BF_W1K = BF_W1T + (size_t)IN * HID;
constexpr size_t BF_W2T = BF_W1K + (size_t)IN * HID, BF_W2K = BF_W2T + (size_t)HID * HID;
constexpr size_t BF_W3T = BF_W2K + (size_t)HID * HID, BF_W3K = BF_W3T + (size_t)HID * OUT;
constexpr size_t NBF16 = BF_W3K + (size_t)HID * OUT;

template <class T>
wc_status dalloc(T** p, size_t count) {
    *p = nullptr;
    if (!count) return WC_OK;
    WC_TRY(::wc::device_alloc(reinterpret_cast<void**>(p), count * sizeof(T)));
    return WC_OK;
}
template <class T>
void dfree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

inline unsigned blocks_for(size_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

// ---- inputs ----------------------------------------------------------------------------------

struct FeatureScales {
    float inv_a, inv_v, dt;
};

// The 19 inputs of one particle (sorted slot i of the judge step) into x[0..IN).
__device__ __forceinline__ void particle_inputs(const SceneConsts& c, const FeatureScales& fs, float4 p, float4 v,
                                                float4 a, float4 jr, float x[IN]) {
    const float rho = p.w;
    const float inv_rho = rho > 0.f ? 1.f / rho : 0.f;
    x[0] = a.x * fs.inv_a;
    x[1] = a.y * fs.inv_a;
    x[2] = a.z * fs.inv_a;
    x[3] = jr.x * fs.dt * fs.inv_a;
    x[4] = jr.y * fs.dt * fs.inv_a;
    x[5] = jr.z * fs.dt * fs.inv_a;
    x[6] = 100.f * jr.w * fs.dt * inv_rho;
    x[7] = v.x * fs.inv_v;
    x[8] = v.y * fs.inv_v;
    x[9] = v.z * fs.inv_v;
    x[10] = rho / c.rho0 - 1.f;
    x[11] = c.k > 0.f ? v.w / (c.k * c.rho0) : 0.f;
    const float inv_h = 1.f / c.h;
    const float wd[6] = {p.x, c.size - p.x, p.y, c.size - p.y, p.z, c.size - p.z};
#pragma unroll
    for (int q = 0; q < 6; ++q) x[12 + q] = fminf(fmaxf(wd[q] * inv_h, 0.f), 1.f);
    x[18] = 100.f * c.k / c.rho0;
#pragma unroll
    for (int q = (int)IN_USED; q < (int)IN; ++q) x[q] = 0.f;
#pragma unroll
    for (int q = 0; q < (int)IN_USED; ++q)
        if (!isfinite(x[q])) x[q] = 0.f;  // an unevaluated (overfull) cell's particles
}

// Constants of the scene that owns particle slot i (batches: binary search in poff).
template <bool BATCHED>
__device__ __forceinline__ const SceneConsts& scene_of(const SceneConsts& sc, const BatchTables& bt, uint32_t i,
                                                       SceneConsts& tmp) {
    if (!BATCHED) return sc;
    tmp = bt.scenes[find_scene(bt.poff, bt.num_scenes, i)];
    return tmp;
}

struct InputSrc {
    const float4 *pos, *vel, *acc, *feat;  // judge step: sorted buffer B, acceleration, J and rate
    SceneConsts sc;
    BatchTables bt;
    FeatureScales fs;
};

// Inputs of every particle as a BF16 matrix [n x IN] (sample recording).
template <bool BATCHED>
__global__ void inputs_kernel(uint32_t n, const InputSrc src, const uint32_t* __restrict__ ids,
                              __nv_bfloat16* __restrict__ out_by_id) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    SceneConsts tmp;
    const SceneConsts& c = scene_of<BATCHED>(src.sc, src.bt, i, tmp);
    float x[IN];
    particle_inputs(c, src.fs, src.pos[i], src.vel[i], src.acc[i], src.feat[i], x);
    const uint32_t row = ids ? ids[i] : i;
    uint4* o = reinterpret_cast<uint4*>(out_by_id + (size_t)row * IN);
#pragma unroll
    for (int q = 0; q < (int)IN / 8; ++q) {
        uint32_t w[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const __nv_bfloat162 b = __floats2bfloat162_rn(x[8 * q + 2 * e], x[8 * q + 2 * e + 1]);
            w[e] = *reinterpret_cast<const uint32_t*>(&b);
        }
        o[q] = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

// ---- skipped steps -------------------------------------------------------------------------------

// The `ages` skipped steps of one particle after a judge step, in registers: v += (a + change_k)
// dt, speed clamp, x += v dt, wall collision (update.comp:191-231) for k = 1 .. ages; then the
// carried density rho_t + (ages + 1) dt rhodot (the density rate of the judge step) and its
// pressure. change = null: the stale acceleration (the method without the network).
__device__ __forceinline__ void skip_particle(const SceneConsts& c, float dt, uint32_t ages, float4 a,
                                              const float* change, float rho_t, float rhodot, float4& p, float4& v) {
    float x[3] = {p.x, p.y, p.z}, u[3] = {v.x, v.y, v.z};
    const float a0[3] = {a.x, a.y, a.z};
#pragma unroll
    for (uint32_t k = 1; k <= MAX_AGES; ++k) {
        if (k > ages) break;
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const float aq = change ? a0[q] + change[3 * (k - 1) + q] : a0[q];
            float va = u[q] + aq * dt;
            if (c.flags & WC_FLAG_SPEED_CLAMP) va = fminf(fmaxf(va, -c.max_speed), c.max_speed);
            float xa = x[q] + va * dt;
            if (xa < c.border) {
                va *= -c.damping;
                xa = c.border;
            } else if (xa > c.size - c.border) {
                va *= -c.damping;
                xa = c.size - c.border;
            }
            x[q] = xa;
            u[q] = va;
        }
    }
    const float rho = rho_t + (float)(ages + 1u) * dt * rhodot;
    float pressure;
    if (c.eos == WC_EOS_LINEAR) {
        pressure = c.p0 + c.k * (rho - c.rho0);
    } else {
        const float r = rho / c.rho0;
        pressure = c.p0 + c.k * (r * r * r - 1.f);
    }
    p = make_float4(x[0], x[1], x[2], rho);
    v = make_float4(u[0], u[1], u[2], pressure);
}

// Where the skipped steps of a cycle read and write: the state buffer after the judge step (in
// the judge step's sorted order), the judge step's acceleration and features, and the slot that
// keeps the state after the judge step for a revert.
struct SkipArgs {
    float4 *pos, *vel;  // pos.w after the judge step: its SPH density (rho_t)
    const float4 *acc, *feat;
    float4 *save_pos, *save_vel;
    const uint32_t* ids;
    uint32_t* save_ids;
    float dt;
    uint32_t ages;
    uint32_t taylor;  // add k dt J (the judge step's J, feat.xyz) to the acceleration of age k
};

// The skipped steps of a cycle: the acceleration of age k is the judge step's, plus k dt J when
// k.taylor is set, plus the network's residual change[i * ldc + 3 (k - 1) ..] when change is
// given, less the residuals' mean over the particles, mean[0 .. 3 ages) (the changes of internal
// forces sum to zero, and a common offset would move every particle the same way).
template <bool BATCHED>
__global__ void skip_cycle_kernel(uint32_t n, const SceneConsts sc0, const BatchTables bt, const SkipArgs k,
                                  const float* __restrict__ change, uint32_t ldc, const float* __restrict__ mean) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    SceneConsts tmp;
    const SceneConsts& c = scene_of<BATCHED>(sc0, bt, i, tmp);
    float4 p = k.pos[i], v = k.vel[i];
    k.save_pos[i] = p;
    k.save_vel[i] = v;
    if (k.ids) k.save_ids[i] = k.ids[i];
    const float4 jf = k.feat[i];
    float ch[3 * MAX_AGES];
#pragma unroll
    for (uint32_t j = 0; j < 3 * MAX_AGES; ++j) {
        const uint32_t age = j / 3u + 1u;
        const float jq = (j % 3u) == 0 ? jf.x : ((j % 3u) == 1 ? jf.y : jf.z);
        float x = k.taylor ? (float)age * k.dt * jq : 0.f;
        if (change && j < 3u * k.ages) x += change[(size_t)i * ldc + j] - mean[j];
        ch[j] = x;
    }
    skip_particle(c, k.dt, k.ages, k.acc[i], (change || k.taylor) ? ch : nullptr, p.w, jf.w, p, v);
    k.pos[i] = p;
    k.vel[i] = v;
}

// ---- fused per-particle network on the tensor cores -------------------------------------------

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// K-major core-matrix layout without swizzle: 8-row x 16-byte core matrices, the next along K
// 128 B away (LBO), the next 8-row group (K / 8) x 128 B away (SBO).
__device__ __forceinline__ uint32_t core_off(uint32_t r, uint32_t k, uint32_t K) {
    return (((r >> 3) * (K >> 3) + (k >> 3)) << 7) + ((r & 7u) << 4) + ((k & 7u) << 1);
}
__device__ __forceinline__ uint64_t core_desc(uint32_t saddr, uint32_t K) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)(128u >> 4) << 16;
    d |= (uint64_t)(((K >> 3) * 128u) >> 4) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}
// kind::f16 instruction descriptor: FP32 accumulator, BF16 A and B, both K-major, M = 128.
__host__ __device__ constexpr uint32_t idesc(uint32_t N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((TILE >> 4) << 24);
}

__device__ __forceinline__ bool mbar_wait(uint32_t addr, uint32_t parity) {
    for (uint32_t i = 0; i < WAIT_LIMIT; ++i) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(addr), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// One row of 8 consecutive K values (16 bytes) of a core-matrix tile.
__device__ __forceinline__ void put8(unsigned char* tile, uint32_t r, uint32_t k, uint32_t K, const float* v) {
    uint32_t w[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
        const __nv_bfloat162 b = __floats2bfloat162_rn(v[2 * e], v[2 * e + 1]);
        w[e] = *reinterpret_cast<const uint32_t*>(&b);
    }
    *reinterpret_cast<uint4*>(tile + core_off(r, k, K)) = make_uint4(w[0], w[1], w[2], w[3]);
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float x[32]) {
    uint32_t v[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
          "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]),
          "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
          "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 32; ++j) x[j] = __uint_as_float(v[j]);
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float x[16]) {
    uint32_t v[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
          "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; ++j) x[j] = __uint_as_float(v[j]);
}

struct MlpWeights {
    const __nv_bfloat16 *w1t, *w2t, *w3t;  // W^T [n_out x k_in], BF16
    const float *b1, *b2, *b3;
};

struct __align__(1024) MlpSmem {
    // the inputs [128 x 32] occupy the first 8 KB of the hidden tile: layer 1's MMAs have read
    // them (their commit arrived) before its epilogue writes the hidden activations
    union {
        unsigned char x[TILE * IN * 2];
        unsigned char h[TILE * HID * 2];  // 16 KB
    };
    unsigned char w1[HID * IN * 2];     // 4 KB
    unsigned char w2[HID * HID * 2];    // 8 KB
    unsigned char w3[OUT * HID * 2];    // 2 KB
    float b1[HID], b2[HID], b3[OUT];
};

// Issue the MMAs of one layer (K / 16 of them) from one thread and commit them to `mbar`.
__device__ __forceinline__ void mma_layer(uint32_t tmem, uint32_t a_base, uint32_t b_base, uint32_t K, uint32_t N,
                                          uint32_t mbar) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    for (uint32_t j = 0; j < K / 16u; ++j) {
        const uint64_t ad = core_desc(a_base + 256u * j, K);
        const uint64_t bd = core_desc(b_base + 256u * j, K);
        const uint32_t acc = j > 0 ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc(N)), "r"(acc));
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

// out[row * ldo + j] = out_scale * y_j for j < nout (rows < n). FUSED: the inputs are computed
// from the judge step's buffers (src); otherwise they are rows of x_in [n x IN] (BF16). SUMS: also
// the CTA's column sums of the outputs, part[blockIdx.x * OUT + j] (tiles and warps added in a
// fixed order, so the sums are reproducible).
template <bool FUSED, bool BATCHED, bool SUMS = false>
__global__ void __launch_bounds__(MLP_THREADS, MLP_CTAS_PER_SM) mlp_kernel(uint32_t n, const InputSrc src,
                                                          const __nv_bfloat16* __restrict__ x_in,
                                                          const MlpWeights wts, float* __restrict__ out, uint32_t ldo,
                                                          uint32_t nout, float out_scale, uint32_t* __restrict__ err,
                                                          float* __restrict__ part = nullptr) {
    __shared__ MlpSmem sm;
    __shared__ float sm_sums[MLP_THREADS / 32][OUT];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    __shared__ int s_failed;
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;

    // weights and biases, once per CTA, into the core-matrix layout
    for (uint32_t id = tid; id < HID * IN / 8; id += MLP_THREADS) {
        const uint32_t r = id / (IN / 8), g = id % (IN / 8);
        *reinterpret_cast<uint4*>(sm.w1 + core_off(r, 8u * g, IN)) =
            __ldg(reinterpret_cast<const uint4*>(wts.w1t + (size_t)r * IN + 8u * g));
    }
    for (uint32_t id = tid; id < HID * HID / 8; id += MLP_THREADS) {
        const uint32_t r = id / (HID / 8), g = id % (HID / 8);
        *reinterpret_cast<uint4*>(sm.w2 + core_off(r, 8u * g, HID)) =
            __ldg(reinterpret_cast<const uint4*>(wts.w2t + (size_t)r * HID + 8u * g));
    }
    for (uint32_t id = tid; id < OUT * HID / 8; id += MLP_THREADS) {
        const uint32_t r = id / (HID / 8), g = id % (HID / 8);
        *reinterpret_cast<uint4*>(sm.w3 + core_off(r, 8u * g, HID)) =
            __ldg(reinterpret_cast<const uint4*>(wts.w3t + (size_t)r * HID + 8u * g));
    }
    for (uint32_t j = tid; j < HID; j += MLP_THREADS) {
        sm.b1[j] = wts.b1[j];
        sm.b2[j] = wts.b2[j];
    }
    if (tid < OUT) sm.b3[tid] = wts.b3[tid];
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&mbar)));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_failed = 0;
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_slot)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;
    const uint32_t tlane = tmem + ((32u * warp) << 16);  // this warp's 32 accumulator rows
    const uint32_t mb = smem_addr(&mbar);
    uint32_t phase = 0;
    const uint32_t ntiles = (n + TILE - 1) / TILE;
    float cta_sum = 0.f;  // thread j < OUT: column j over this CTA's tiles
    // FUSED: this thread's row of the next tile, loaded one tile ahead so that the loads overlap
    // the current tile's MMAs
    float4 nx_p = make_float4(0.f, 0.f, 0.f, 0.f), nx_v = nx_p, nx_a = nx_p, nx_f = nx_p;
    if (FUSED && (size_t)blockIdx.x * TILE + tid < n) {
        const uint32_t r = blockIdx.x * TILE + tid;
        nx_p = src.pos[r];
        nx_v = src.vel[r];
        nx_a = src.acc[r];
        nx_f = src.feat[r];
    }

    for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const uint32_t row = tile * TILE + tid;
        const bool valid = row < n;
        {
            float x[IN];
            if (FUSED) {
                const float4 cp = nx_p, cv = nx_v, ca = nx_a, cf = nx_f;
                const size_t next = (size_t)(tile + gridDim.x) * TILE + tid;
                if (next < n) {
                    nx_p = src.pos[next];
                    nx_v = src.vel[next];
                    nx_a = src.acc[next];
                    nx_f = src.feat[next];
                }
                if (valid) {
                    SceneConsts tmp;
                    const SceneConsts& c = scene_of<BATCHED>(src.sc, src.bt, row, tmp);
                    particle_inputs(c, src.fs, cp, cv, ca, cf, x);
                } else {
#pragma unroll
                    for (int q = 0; q < (int)IN; ++q) x[q] = 0.f;
                }
#pragma unroll
                for (uint32_t g = 0; g < IN / 8; ++g) put8(sm.x, tid, 8u * g, IN, x + 8 * g);
            } else {
#pragma unroll
                for (uint32_t g = 0; g < IN / 8; ++g) {
                    uint4 v = make_uint4(0u, 0u, 0u, 0u);
                    if (valid) v = __ldg(reinterpret_cast<const uint4*>(x_in + (size_t)row * IN) + g);
                    *reinterpret_cast<uint4*>(sm.x + core_off(tid, 8u * g, IN)) = v;
                }
            }
        }
        // layer 1: [128 x 32] . W1 -> 64 accumulator columns
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0 && !s_failed) mma_layer(tmem, smem_addr(sm.x), smem_addr(sm.w1), IN, HID, mb);
        bool ok = s_failed ? false : mbar_wait(mb, phase);
        phase ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        for (uint32_t c0 = 0; c0 < HID; c0 += 32) {
            float y[32];
            tmem_ld32(tlane + c0, y);
#pragma unroll
            for (int j = 0; j < 32; ++j) y[j] = fmaxf(y[j] + sm.b1[c0 + j], 0.f);
#pragma unroll
            for (uint32_t g = 0; g < 4; ++g) put8(sm.h, tid, c0 + 8u * g, HID, y + 8 * g);
        }
        if (!ok) atomicOr(&s_failed, 1);
        // layer 2: [128 x 64] . W2 -> 64 columns (the accumulator is free: its loads have waited)
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0 && !s_failed) mma_layer(tmem, smem_addr(sm.h), smem_addr(sm.w2), HID, HID, mb);
        ok = s_failed ? false : mbar_wait(mb, phase);
        phase ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // the MMAs have read all of h1 (their commit arrived): h2 overwrites it, 32 columns at a
        // time (each thread writes its own row only)
        for (uint32_t c0 = 0; c0 < HID; c0 += 32) {
            float y[32];
            tmem_ld32(tlane + c0, y);
#pragma unroll
            for (int j = 0; j < 32; ++j) y[j] = fmaxf(y[j] + sm.b2[c0 + j], 0.f);
#pragma unroll
            for (uint32_t g = 0; g < 4; ++g) put8(sm.h, tid, c0 + 8u * g, HID, y + 8 * g);
        }
        if (!ok) atomicOr(&s_failed, 1);
        // layer 3: [128 x 64] . W3 -> 16 columns
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0 && !s_failed) mma_layer(tmem, smem_addr(sm.h), smem_addr(sm.w3), HID, OUT, mb);
        ok = s_failed ? false : mbar_wait(mb, phase);
        phase ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        {
            float y[16];
            tmem_ld16(tlane, y);
#pragma unroll
            for (uint32_t j = 0; j < OUT; ++j) y[j] = (valid && ok && j < nout) ? out_scale * (y[j] + sm.b3[j]) : 0.f;
            if (valid && ok) {
                float* o = out + (size_t)row * ldo;
                if ((ldo & 3u) == 0 && (nout & 3u) == 0) {  // whole 16-byte groups
#pragma unroll
                    for (uint32_t j = 0; j < OUT; j += 4)
                        if (j < nout) *reinterpret_cast<float4*>(o + j) = make_float4(y[j], y[j + 1], y[j + 2], y[j + 3]);
                } else {
#pragma unroll
                    for (uint32_t j = 0; j < OUT; ++j)
                        if (j < nout) o[j] = y[j];
                }
            }
            if (SUMS) {
                // the outputs as floats into the hidden tile (layer 3's MMAs have read it), rows
                // 17 floats apart so that a column's 16-row runs hit distinct banks
                float* sy = reinterpret_cast<float*>(sm.h);
#pragma unroll
                for (uint32_t j = 0; j < OUT; ++j) sy[tid * 17u + j] = y[j];
            }
        }
        if (SUMS) {
            __syncthreads();
            // thread 16 g + j adds column j over rows 16 g .. 16 g + 15; the two row groups of a
            // warp meet in one shuffle, the four warps in a fixed order
            const float* sy = reinterpret_cast<const float*>(sm.h);
            const uint32_t g = tid >> 4, jc = tid & 15u;
            float v = 0.f;
#pragma unroll
            for (uint32_t r = 0; r < 16; ++r) v += sy[(16u * g + r) * 17u + jc];
            v += __shfl_xor_sync(0xffffffffu, v, 16);
            if ((lane & 16u) == 0) sm_sums[warp][jc] = v;
            __syncthreads();
            if (tid < OUT) cta_sum += ((sm_sums[0][tid] + sm_sums[1][tid]) + sm_sums[2][tid]) + sm_sums[3][tid];
        }
        if (!ok) atomicOr(&s_failed, 1);
        // the next tile rewrites x and h and the accumulator
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        if (s_failed) break;
    }
    if (s_failed && tid == 0 && err) atomicOr(err, DEVERR_MMA_TIMEOUT);
    if (SUMS && tid < OUT) part[(size_t)blockIdx.x * OUT + tid] = cta_sum;
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
    }
}

// mean[j] = (sum over CTAs of part[cta][j]) / n, j < OUT: one warp per column, FP32 in a fixed
// order (FP64 arithmetic is slow on this GPU and the mean needs no more than FP32).
__global__ void __launch_bounds__(32 * OUT) output_mean_kernel(uint32_t ctas, uint32_t n, const float* __restrict__ part,
                                                               float* __restrict__ mean) {
    const uint32_t j = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    float a = 0.f;
    for (uint32_t c = lane; c < ctas; c += 32u) a += part[(size_t)c * OUT + j];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) a += __shfl_xor_sync(0xffffffffu, a, off);
    if (lane == 0) mean[j] = n ? a / (float)n : 0.f;
}

// ---- rollout kernels ----------------------------------------------------------------------------

// Judge: the judge step's density pass sums |rho_carried / rho_SPH - 1| per chunk of 32 sorted
// slots; this kernel adds the chunk sums in a fixed order, FP32 per thread and warp (a relative
// rounding of order 1e-6 against a tolerance of order 1e-2), FP64 across the warps.
constexpr uint32_t JUDGE_THREADS = 1024;
__global__ void __launch_bounds__(JUDGE_THREADS) judge_final_kernel(uint32_t chunks, const float* __restrict__ part,
                                                                    double* __restrict__ out) {
    __shared__ float s[JUDGE_THREADS / 32];
    float a = 0.f;
    for (uint32_t b = threadIdx.x; b < chunks; b += JUDGE_THREADS) a += part[b];
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) a += __shfl_xor_sync(0xffffffffu, a, off);
    if ((threadIdx.x & 31u) == 0) s[threadIdx.x >> 5] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (uint32_t w = 0; w < JUDGE_THREADS / 32; ++w) t += s[w];
        *out = t;
    }
}

// ---- sample recording ---------------------------------------------------------------------------

// a0_by_id[ids[i]] = acc[i]
// The judge step's acceleration and J by particle id; y_by_id[id][JD .. JD + 2] = dt J / a_s and
// y_by_id[id][RES_SCALE] = (DT_REF / dt)^2.
__global__ void scatter_judge_kernel(uint32_t n, const uint32_t* __restrict__ ids, const float4* __restrict__ acc,
                                     const float4* __restrict__ feat, float dt, float inv_a,
                                     float4* __restrict__ a0_by_id, float4* __restrict__ j0_by_id,
                                     float* __restrict__ y_by_id) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t id = ids[i];
    const float4 j = feat[i];
    a0_by_id[id] = acc[i];
    j0_by_id[id] = j;
    float* y = y_by_id + (size_t)id * YW;
    y[RES_SCALE] = (DT_REF / dt) * (DT_REF / dt);
    y[JD] = j.x * dt * inv_a;
    y[JD + 1] = j.y * dt * inv_a;
    y[JD + 2] = j.z * dt * inv_a;
}
// y_by_id[ids[i]][3 (age - 1) ..] = (acc[i] - a0 - age dt J) * inv_a: the residual of the Taylor
// extrapolation the network learns.
__global__ void target_kernel(uint32_t n, const uint32_t* __restrict__ ids, const float4* __restrict__ acc,
                              const float4* __restrict__ a0_by_id, const float4* __restrict__ j0_by_id, uint32_t age,
                              float dt, float inv_a, float* __restrict__ y_by_id) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t id = ids[i];
    const float4 a = acc[i], b = a0_by_id[id], j = j0_by_id[id];
    const float kdt = (float)age * dt;
    float* y = y_by_id + (size_t)id * YW + 3u * (age - 1u);
    y[0] = (a.x - fmaf(kdt, j.x, b.x)) * inv_a;
    y[1] = (a.y - fmaf(kdt, j.y, b.y)) * inv_a;
    y[2] = (a.z - fmaf(kdt, j.z, b.z)) * inv_a;
}

// ---- training -------------------------------------------------------------------------------------

inline uint64_t splitmix64(uint64_t& st) {
    uint64_t z = (st += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
// rows of the minibatch: idx ? idx[r] : a draw in [0, count) from the step's seed
__global__ void gather_rows_kernel(uint32_t rows, uint64_t seed, uint64_t count, const uint32_t* __restrict__ idx,
                                   const __nv_bfloat16* __restrict__ xs, const float* __restrict__ ys,
                                   __nv_bfloat16* __restrict__ xb, float* __restrict__ yb) {
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    const uint64_t k = idx ? (uint64_t)idx[r] % count : mix64(seed + 0x9E3779B97F4A7C15ull * (r + 1ull)) % count;
    const uint4* sx = reinterpret_cast<const uint4*>(xs + k * IN);
    uint4* dx = reinterpret_cast<uint4*>(xb + (size_t)r * IN);
#pragma unroll
    for (int q = 0; q < (int)IN / 8; ++q) dx[q] = sx[q];
    // the residuals in the network's units: times (DT_REF / dt)^2 (column RES_SCALE)
    const float* sy = ys + k * YW;
    const float sc = sy[RES_SCALE];
    float* dy = yb + (size_t)r * OUT;
#pragma unroll
    for (int q = 0; q < (int)OUT; ++q) dy[q] = q < (int)(3 * MAX_AGES) ? sy[q] * sc : 0.f;
}

// Mean squared error over the used outputs: d = 2 (p - t) / (rows nout) (FP32 and BF16, unused
// columns zero) and per-block partial sums of the squared error.
__global__ void __launch_bounds__(256) loss_kernel(uint32_t rows, uint32_t nout, const float* __restrict__ pred,
                                                   const float* __restrict__ tgt, float* __restrict__ d32,
                                                   __nv_bfloat16* __restrict__ d16, float* __restrict__ part) {
    __shared__ float s[256];
    const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
    float acc = 0.f;
    if (r < rows) {
        const float scale = 2.f / ((float)rows * (float)nout);
#pragma unroll
        for (uint32_t j = 0; j < OUT; ++j) {
            float d = 0.f;
            if (j < nout) {
                const float e = pred[(size_t)r * OUT + j] - tgt[(size_t)r * OUT + j];
                acc += e * e;
                d = scale * e;
            }
            d32[(size_t)r * OUT + j] = d;
            d16[(size_t)r * OUT + j] = __float2bfloat16_rn(d);
        }
    }
    s[threadIdx.x] = acc;
    __syncthreads();
    for (uint32_t h = 128; h > 0; h >>= 1) {
        if (threadIdx.x < h) s[threadIdx.x] += s[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = s[0];
}

// split-K partials [splits][m x n] -> out (fixed order)
__global__ void reduce_splits_kernel(uint32_t count, uint32_t splits, const float* __restrict__ part,
                                     float* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    float a = 0.f;
    for (uint32_t s = 0; s < splits; ++s) a += part[(size_t)s * count + i];
    out[i] = a;
}

// Evaluation sums per age k (units of a_s; y the residual, jd = dt J from the targets' columns
// JD .., a0 from the inputs' first three columns, pred converted from the network's units):
// |pred - y|^2 (network mode),
// |y + k jd|^2 (stale mode), |y|^2 (Taylor mode), |a0 + y + k jd|^2 (the acceleration).
constexpr uint32_t EVAL_SUMS = 4;
__global__ void eval_kernel(uint64_t rows, uint32_t ages, const __nv_bfloat16* __restrict__ xs,
                            const float* __restrict__ ys, const float* __restrict__ pred, double* __restrict__ part) {
    __shared__ double s[EVAL_SUMS * MAX_AGES][128];
    const uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    double acc[EVAL_SUMS * MAX_AGES];
#pragma unroll
    for (int q = 0; q < (int)(EVAL_SUMS * MAX_AGES); ++q) acc[q] = 0.0;
    if (r < rows) {
        const float a0[3] = {__bfloat162float(xs[r * IN + 0]), __bfloat162float(xs[r * IN + 1]),
                             __bfloat162float(xs[r * IN + 2])};
        for (uint32_t g = 0; g < ages; ++g) {
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const double y = ys[r * YW + 3 * g + c];
                const double p = pred[r * OUT + 3 * g + c] / (double)ys[r * YW + RES_SCALE];
                const double ch = y + (double)(g + 1) * ys[r * YW + JD + c];
                const double t = a0[c] + ch;
                acc[EVAL_SUMS * g + 0] += (p - y) * (p - y);
                acc[EVAL_SUMS * g + 1] += ch * ch;
                acc[EVAL_SUMS * g + 2] += y * y;
                acc[EVAL_SUMS * g + 3] += t * t;
            }
        }
    }
#pragma unroll
    for (int q = 0; q < (int)(EVAL_SUMS * MAX_AGES); ++q) s[q][threadIdx.x] = acc[q];
    __syncthreads();
    for (uint32_t h = 64; h > 0; h >>= 1) {
        if (threadIdx.x < h)
            for (int q = 0; q < (int)(EVAL_SUMS * MAX_AGES); ++q) s[q][threadIdx.x] += s[q][threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int q = 0; q < (int)(EVAL_SUMS * MAX_AGES); ++q)
            part[(size_t)blockIdx.x * EVAL_SUMS * MAX_AGES + q] = s[q][0];
}

}  // namespace

struct wc_local {
    wc_local_config cfg{};
    float *w = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;  // FP32 master, gradient, Adam moments
    __nv_bfloat16* wb = nullptr;                                    // BF16 copies (NBF16)
    int adam_step = 0;
    bool cast_dirty = true;
    cudaStream_t stream = nullptr;
    uint32_t* d_err = nullptr;
    uint32_t* h_err = nullptr;
    int sms = 1;
    // samples: inputs [cap x IN] BF16, targets [cap x OUT] FP32 (train, held out)
    __nv_bfloat16* xs[2] = {nullptr, nullptr};
    float* ys[2] = {nullptr, nullptr};
    uint64_t cap[2] = {0, 0}, count[2] = {0, 0};
    // recording scratch (by particle id)
    __nv_bfloat16* x_id = nullptr;
    float* y_id = nullptr;
    float4* a0_id = nullptr;
    float4* j0_id = nullptr;  // the judge step's J by particle id (recording)
    float4* feat = nullptr;   // judge step: (J, density rate) per sorted slot
    float2* rate = nullptr;   // judge step's density pass: (density rate, pressure rate) per sorted slot
    uint32_t cap_n = 0;
    // training scratch
    uint32_t cap_rows = 0;
    __nv_bfloat16 *xb = nullptr, *h1 = nullptr, *h2 = nullptr, *dy16 = nullptr, *dz16 = nullptr;
    float *yb = nullptr, *yp = nullptr, *dy32 = nullptr, *dh = nullptr, *part = nullptr, *loss_part = nullptr;
    size_t part_cap = 0;
    float* colsum_part = nullptr;
    // rollout scratch
    float* change = nullptr;
    float* mean_part = nullptr;  // per-CTA column sums of the network's outputs
    float* mean = nullptr;       // their mean over the particles [OUT]
    float* vxyz = nullptr;  // judge steps: the gather's sorted velocities (x, y, z arrays)
    float4 *save_pos[2] = {nullptr, nullptr}, *save_vel[2] = {nullptr, nullptr};
    uint32_t* save_ids[2] = {nullptr, nullptr};
    float* judge_part = nullptr;  // per chunk of 32 sorted slots
    double *judge_out = nullptr, *h_judge = nullptr;
    uint32_t cap_roll = 0;
};

namespace {

void free_local(wc_local* s) {
    dfree(s->w);
    dfree(s->g);
    dfree(s->m);
    dfree(s->v);
    dfree(s->wb);
    dfree(s->d_err);
    for (int q = 0; q < 2; ++q) {
        dfree(s->xs[q]);
        dfree(s->ys[q]);
        dfree(s->save_pos[q]);
        dfree(s->save_vel[q]);
        dfree(s->save_ids[q]);
    }
    dfree(s->x_id);
    dfree(s->y_id);
    dfree(s->a0_id);
    dfree(s->j0_id);
    dfree(s->feat);
    dfree(s->rate);
    dfree(s->xb);
    dfree(s->h1);
    dfree(s->h2);
    dfree(s->dy16);
    dfree(s->dz16);
    dfree(s->yb);
    dfree(s->yp);
    dfree(s->dy32);
    dfree(s->dh);
    dfree(s->part);
    dfree(s->loss_part);
    dfree(s->colsum_part);
    dfree(s->change);
    dfree(s->mean_part);
    dfree(s->mean);
    dfree(s->vxyz);
    dfree(s->judge_part);
    dfree(s->judge_out);
    if (s->h_err) cudaFreeHost(s->h_err);
    if (s->h_judge) cudaFreeHost(s->h_judge);
    if (s->stream) cudaStreamDestroy(s->stream);
}

wc_status read_err(wc_local* s) {
    WC_CUDA_TRY(cudaGetLastError());
    WC_CUDA_TRY(cudaMemcpyAsync(s->h_err, s->d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream));
    WC_CUDA_TRY(cudaStreamSynchronize(s->stream));
    if (*s->h_err) {
        *s->h_err = 0;
        WC_CUDA_TRY(cudaMemsetAsync(s->d_err, 0, sizeof(uint32_t), s->stream));
        return fail(WC_ERR_TIMEOUT, "a tensor-core wait of the learned rollout's network exceeded its limit");
    }
    return WC_OK;
}

void cast(wc_local* s) {
    if (!s->cast_dirty) return;
    nn::cast_weight(s->w + OFF_W1, IN, HID, IN, HID, s->wb + BF_W1T, s->wb + BF_W1K, s->stream);
    nn::cast_weight(s->w + OFF_W2, HID, HID, HID, HID, s->wb + BF_W2T, s->wb + BF_W2K, s->stream);
    nn::cast_weight(s->w + OFF_W3, HID, OUT, HID, OUT, s->wb + BF_W3T, s->wb + BF_W3K, s->stream);
    s->cast_dirty = false;
}

MlpWeights weights(const wc_local* s) {
    return MlpWeights{s->wb + BF_W1T, s->wb + BF_W2T, s->wb + BF_W3T, s->w + OFF_B1, s->w + OFF_B2, s->w + OFF_B3};
}

// Persistent grid of the network kernel: MLP_CTAS_PER_SM CTAs on every SM, at most one per tile.
// The kernel is latency-bound (three MMA round trips per tile), so every SM runs as many tiles at
// once as fit: __launch_bounds__(128, 6) holds a thread to 85 registers, a CTA takes 32 KB of
// shared memory and 64 of the SM's 512 tensor-memory columns.
int mlp_grid(const wc_local* s, uint32_t n) {
    const uint32_t tiles = (n + TILE - 1) / TILE;
    const uint32_t g = std::min<uint32_t>(tiles, (uint32_t)s->sms * MLP_CTAS_PER_SM);
    return (int)std::max(1u, g);
}

InputSrc input_src(const wc_local* s, const StepTarget& t, float dt) {
    InputSrc src{};
    src.pos = t.d->pos_b;
    src.vel = t.d->vel_b;
    src.acc = t.d->accel;
    src.feat = s->feat;
    src.sc = t.sc;
    src.bt = t.bt;
    (void)dt;
    src.fs = FeatureScales{1.f / s->cfg.accel_scale, 1.f / s->cfg.velocity_scale, DT_REF};
    return src;
}

// The network's outputs -> m/s^2 at time step dt: a_s (dt / DT_REF)^2.
float residual_scale(const wc_local* s, float dt) { return s->cfg.accel_scale * (dt / DT_REF) * (dt / DT_REF); }

// The network on the judge step's buffers -> s->change [n x 4 ages] (accelerations, m/s^2).
void enqueue_predict(wc_local* s, const StepTarget& t, float dt) {
    const uint32_t n = t.d->n;
    if (!n) return;
    cast(s);
    const InputSrc src = input_src(s, t, dt);
    const uint32_t ldo = 3u * s->cfg.ages;
    if (t.bt.num_scenes)
        mlp_kernel<true, true><<<mlp_grid(s, n), MLP_THREADS, 0, s->stream>>>(
            n, src, nullptr, weights(s), s->change, ldo, ldo, residual_scale(s, dt), s->d_err);
    else
        mlp_kernel<true, false><<<mlp_grid(s, n), MLP_THREADS, 0, s->stream>>>(
            n, src, nullptr, weights(s), s->change, ldo, ldo, residual_scale(s, dt), s->d_err);
}

// The judge of the last cycle when the rollout ends after its skipped steps: the sort and the
// judge step's density pass with its judge sums, without a force pass (the state does not
// advance).
void enqueue_closing_judge(wc_local* s, const StepTarget& t) {
    DevBuffers& d = *t.d;
    if (!d.n) return;
    if (t.bt.num_scenes)
        launch_bin_count_batched(d, t.bt, t.ld, t.stream);
    else
        launch_bin_count(d, t.sc, t.ld, t.stream);
    launch_scan_cells(d, t.stream);
    launch_scatter(d, t.ld, t.stream);
    launch_rank_gather(d, t.ld, t.stream);
    if (t.bt.num_scenes)
        launch_density_batched_feat(d, t.bt, t.ld, FEAT_RATE, nullptr, nullptr, s->judge_part, t.stream);
    else
        launch_density_feat(d, t.sc, t.ld, FEAT_RATE, nullptr, nullptr, s->judge_part, t.stream);
    judge_final_kernel<<<1, JUDGE_THREADS, 0, t.stream>>>(blocks_for(d.n, 32), s->judge_part, s->judge_out);
}

// The judge step, on the target's stream: a plain SPH step whose force pass also writes s->feat
// (feature level FEAT_RATE: the density rate in .w; FEAT_FULL: also J, from the density pass's
// rates in s->rate). With `judge`, the density pass also sums |rho_carried / rho_SPH - 1| (the
// sorted buffer's densities before the pass are the ones the skipped steps carried) and the final
// sum follows it.
void enqueue_judge_step(wc_local* s, const StepTarget& t, float dt, bool judge, int level = FEAT_FULL) {
    DevBuffers& d = *t.d;
    StepInputs in = *t.in;
    in.dt = dt;
    if (t.bt.num_scenes) {
        launch_bin_count_batched(d, t.bt, t.ld, t.stream);
    } else {
        launch_bin_count(d, t.sc, t.ld, t.stream);
    }
    launch_scan_cells(d, t.stream);
    launch_scatter(d, t.ld, t.stream);
    const bool full = level == FEAT_FULL;
    launch_rank_gather(d, t.ld, t.stream, full ? s->vxyz : nullptr);
    const FeatureBuffers fb{s->feat, s->rate};
    float* jp = judge && d.n ? s->judge_part : nullptr;
    if (t.bt.num_scenes) {
        launch_density_batched_feat(d, t.bt, t.ld, level, s->vxyz, s->rate, jp, t.stream);
        launch_force_batched_feat(d, t.bt, in, t.ld, level, fb, t.stream);
    } else {
        launch_density_feat(d, t.sc, t.ld, level, s->vxyz, s->rate, jp, t.stream);
        launch_force_feat(d, t.sc, in, t.ld, level, fb, t.stream);
    }
    if (jp) judge_final_kernel<<<1, JUDGE_THREADS, 0, t.stream>>>(blocks_for(d.n, 32), jp, s->judge_out);
}

wc_status plain_step(const StepTarget& t, float dt) {
    return t.fluid ? fluid_graph_step(t.fluid, dt) : batch_graph_step(t.batch, dt);
}

wc_status set_recording(const StepTarget& t, bool on) {
    return t.fluid ? wc_fluid_set_recording(t.fluid, on ? 1 : 0) : wc_batch_set_recording(t.batch, on ? 1 : 0);
}

wc_status target_check(const StepTarget& t) { return t.fluid ? fluid_check(t.fluid) : batch_check(t.batch); }

wc_status ensure_n(wc_local* s, uint32_t n) {
    if (n <= s->cap_n) return WC_OK;
    dfree(s->x_id);
    dfree(s->y_id);
    dfree(s->a0_id);
    dfree(s->j0_id);
    dfree(s->feat);
    dfree(s->rate);
    dfree(s->vxyz);
    s->cap_n = 0;
    WC_TRY(dalloc(&s->x_id, (size_t)n * IN));
    WC_TRY(dalloc(&s->y_id, (size_t)n * YW));
    WC_TRY(dalloc(&s->a0_id, n));
    WC_TRY(dalloc(&s->j0_id, n));
    WC_TRY(dalloc(&s->feat, n));
    WC_TRY(dalloc(&s->rate, n));
    WC_TRY(dalloc(&s->vxyz, 3 * (size_t)xyz_stride_for(n)));
    s->cap_n = n;
    return WC_OK;
}

wc_status ensure_samples(wc_local* s, int set) {
    if (s->xs[set]) return WC_OK;
    const uint64_t cap = set == 0 ? s->cfg.capacity : std::max<uint64_t>(s->cfg.capacity / 4, 1);
    WC_TRY(dalloc(&s->xs[set], cap * IN));
    WC_TRY(dalloc(&s->ys[set], cap * YW));
    s->cap[set] = cap;
    s->count[set] = 0;
    return WC_OK;
}

// Cycles of plain SPH on t, recording samples into set `set`.
wc_status record(wc_local* s, const StepTarget& t0, float dt, uint32_t cycles, int set) {
    StepTarget t = t0;
    const uint32_t n = t.d->n;
    if (!t.d->ids_a || !t.d->ids_b) return fail(WC_ERR_STATE, "recording samples needs particle ids (WC_FLAG_TRACK_IDS)");
    WC_TRY(ensure_n(s, n));
    WC_TRY(ensure_samples(s, set));
    const bool had_accel = t.d->accel != nullptr;
    if (!had_accel) WC_TRY(set_recording(t, true));
    t.ld = t0.fluid ? fluid_target(t0.fluid).ld : batch_target(t0.batch).ld;
    const uint32_t ages = s->cfg.ages;
    const FeatureScales fs{1.f / s->cfg.accel_scale, 1.f / s->cfg.velocity_scale, DT_REF};
    wc_status rc = WC_OK;
    for (uint32_t c = 0; c < cycles && rc == WC_OK; ++c) {
        if (s->count[set] + n > s->cap[set]) break;  // full
        enqueue_judge_step(s, t, dt, false);
        InputSrc src = input_src(s, t, dt);
        src.fs = fs;
        if (n) {
            if (t.bt.num_scenes)
                inputs_kernel<true><<<blocks_for(n, 128), 128, 0, t.stream>>>(n, src, t.d->ids_b, s->x_id);
            else
                inputs_kernel<false><<<blocks_for(n, 128), 128, 0, t.stream>>>(n, src, t.d->ids_b, s->x_id);
            cudaMemsetAsync(s->y_id, 0, sizeof(float) * (size_t)n * YW, t.stream);
            scatter_judge_kernel<<<blocks_for(n, 256), 256, 0, t.stream>>>(n, t.d->ids_a, t.d->accel, s->feat, dt,
                                                                          fs.inv_a, s->a0_id, s->j0_id, s->y_id);
        }
        if (t.fluid) fluid_count_step(t.fluid);
        for (uint32_t k = 1; k <= ages && rc == WC_OK; ++k) {
            rc = plain_step(t, dt);
            if (t.fluid) fluid_count_step(t.fluid);
            if (rc == WC_OK && n)
                target_kernel<<<blocks_for(n, 256), 256, 0, t.stream>>>(n, t.d->ids_a, t.d->accel, s->a0_id,
                                                                        s->j0_id, k, dt, fs.inv_a, s->y_id);
        }
        if (rc != WC_OK) break;
        const uint64_t base = s->count[set];
        rc = cudaMemcpyAsync(s->xs[set] + base * IN, s->x_id, sizeof(__nv_bfloat16) * (size_t)n * IN,
                             cudaMemcpyDeviceToDevice, t.stream) == cudaSuccess
                 ? WC_OK
                 : fail(WC_ERR_CUDA, "sample copy failed");
        if (rc == WC_OK)
            rc = cudaMemcpyAsync(s->ys[set] + base * YW, s->y_id, sizeof(float) * (size_t)n * YW,
                                 cudaMemcpyDeviceToDevice, t.stream) == cudaSuccess
                     ? WC_OK
                     : fail(WC_ERR_CUDA, "sample copy failed");
        s->count[set] += n;
    }
    if (rc == WC_OK) rc = target_check(t);
    if (!had_accel) {
        const wc_status r2 = set_recording(t, false);
        if (rc == WC_OK) rc = r2;
    }
    return rc;
}

wc_status ensure_train(wc_local* s, uint32_t rows) {
    if (rows <= s->cap_rows) return WC_OK;
    dfree(s->xb);
    dfree(s->h1);
    dfree(s->h2);
    dfree(s->dy16);
    dfree(s->dz16);
    dfree(s->yb);
    dfree(s->yp);
    dfree(s->dy32);
    dfree(s->dh);
    dfree(s->loss_part);
    dfree(s->colsum_part);
    s->cap_rows = 0;
    WC_TRY(dalloc(&s->xb, (size_t)rows * IN));
    WC_TRY(dalloc(&s->h1, (size_t)rows * HID));
    WC_TRY(dalloc(&s->h2, (size_t)rows * HID));
    WC_TRY(dalloc(&s->dy16, (size_t)rows * OUT));
    WC_TRY(dalloc(&s->dz16, (size_t)rows * HID));
    WC_TRY(dalloc(&s->yb, (size_t)rows * OUT));
    WC_TRY(dalloc(&s->yp, (size_t)rows * OUT));
    WC_TRY(dalloc(&s->dy32, (size_t)rows * OUT));
    WC_TRY(dalloc(&s->dh, (size_t)rows * HID));
    WC_TRY(dalloc(&s->loss_part, blocks_for(rows, 256)));
    WC_TRY(dalloc(&s->colsum_part, (size_t)nn::colsum_blocks(rows) * HID));
    s->cap_rows = rows;
    return WC_OK;
}

wc_status ensure_part(wc_local* s, size_t count) {
    if (count <= s->part_cap) return WC_OK;
    dfree(s->part);
    s->part_cap = 0;
    WC_TRY(dalloc(&s->part, count));
    s->part_cap = count;
    return WC_OK;
}

// C [m x n] (FP32 or BF16) = A . B, see nn::GemmArgs.
wc_status gemm(wc_local* s, uint32_t m, uint32_t n, uint32_t k, const __nv_bfloat16* a, uint32_t lda, int a_t,
               const __nv_bfloat16* b, uint32_t ldb, int b_row, const float* bias, int relu, float* c32,
               __nv_bfloat16* c16, uint32_t ldc) {
    nn::GemmArgs g{};
    g.m = m;
    g.n = n;
    g.k = k;
    g.k_chunk = ((k + 63u) / 64u) * 64u;
    g.a = a;
    g.lda = lda;
    g.a_transposed = a_t;
    g.b = b;
    g.ldb = ldb;
    g.b_rowmajor = b_row;
    g.bias = bias;
    g.relu = relu;
    g.c_f32 = c32;
    g.c_bf16 = c16;
    g.ldc = ldc;
    return nn::launch_gemm(g, s->d_err, s->stream);
}

// Weight gradient dW [kin x nout] = X^T dY over `rows` rows, split over K (rows) in chunks of
// 4,096 and reduced in a fixed order.
wc_status wgrad(wc_local* s, uint32_t rows, const __nv_bfloat16* x, uint32_t kin, const __nv_bfloat16* dy,
                uint32_t nout, float* out) {
    const uint32_t chunk = 4096;
    const uint32_t splits = (rows + chunk - 1) / chunk;
    WC_TRY(ensure_part(s, (size_t)splits * kin * nout));
    nn::GemmArgs g{};
    g.m = kin;
    g.n = nout;
    g.k = rows;
    g.k_chunk = chunk;
    g.a = x;
    g.lda = kin;
    g.a_transposed = 1;
    g.b = dy;
    g.ldb = nout;
    g.b_rowmajor = 1;
    g.c_f32 = s->part;
    g.ldc = nout;
    g.split_stride = (size_t)kin * nout;
    WC_TRY(nn::launch_gemm(g, s->d_err, s->stream));
    const uint32_t cnt = kin * nout;
    reduce_splits_kernel<<<blocks_for(cnt, 256), 256, 0, s->stream>>>(cnt, splits, s->part, out);
    return WC_OK;
}

// Forward and backward over one minibatch (rows drawn from `seed`, or the rows `idx` when set):
// gradients in s->g; with lr > 0 also one Adam step.
wc_status train_step(wc_local* s, uint32_t rows, uint64_t seed, const uint32_t* idx, float lr, float* loss_host) {
    cast(s);
    const uint32_t nout = 3u * s->cfg.ages;
    gather_rows_kernel<<<blocks_for(rows, 256), 256, 0, s->stream>>>(rows, seed, s->count[0], idx, s->xs[0], s->ys[0],
                                                                     s->xb, s->yb);
    // forward
    WC_TRY(gemm(s, rows, HID, IN, s->xb, IN, 0, s->wb + BF_W1T, IN, 0, s->w + OFF_B1, 1, nullptr, s->h1, HID));
    WC_TRY(gemm(s, rows, HID, HID, s->h1, HID, 0, s->wb + BF_W2T, HID, 0, s->w + OFF_B2, 1, nullptr, s->h2, HID));
    WC_TRY(gemm(s, rows, OUT, HID, s->h2, HID, 0, s->wb + BF_W3T, HID, 0, s->w + OFF_B3, 0, s->yp, nullptr, OUT));
    const uint32_t lb = blocks_for(rows, 256);
    loss_kernel<<<lb, 256, 0, s->stream>>>(rows, nout, s->yp, s->yb, s->dy32, s->dy16, s->loss_part);
    // backward: layer 3
    WC_TRY(wgrad(s, rows, s->h2, HID, s->dy16, OUT, s->g + OFF_W3));
    nn::colsum(rows, OUT, OUT, s->dy32, s->colsum_part, s->g + OFF_B3, 0, s->stream);
    WC_TRY(gemm(s, rows, HID, OUT, s->dy16, OUT, 0, s->wb + BF_W3K, OUT, 0, nullptr, 0, s->dh, nullptr, HID));
    nn::relu_mask((size_t)rows * HID, s->dh, s->h2, s->dz16, s->stream);
    // layer 2
    WC_TRY(wgrad(s, rows, s->h1, HID, s->dz16, HID, s->g + OFF_W2));
    nn::colsum(rows, HID, HID, s->dh, s->colsum_part, s->g + OFF_B2, 0, s->stream);
    WC_TRY(gemm(s, rows, HID, HID, s->dz16, HID, 0, s->wb + BF_W2K, HID, 0, nullptr, 0, s->dh, nullptr, HID));
    nn::relu_mask((size_t)rows * HID, s->dh, s->h1, s->dz16, s->stream);
    // layer 1
    WC_TRY(wgrad(s, rows, s->xb, IN, s->dz16, HID, s->g + OFF_W1));
    nn::colsum(rows, HID, HID, s->dh, s->colsum_part, s->g + OFF_B1, 0, s->stream);
    if (lr > 0.f) {
        ++s->adam_step;
        nn::adam(NPARAMS, s->w, s->g, s->m, s->v, lr, 0.9f, 0.999f, 1e-8f, s->adam_step, 1.0f, s->stream);
        s->cast_dirty = true;
    }
    if (loss_host) {
        std::vector<float> parts(lb);
        WC_CUDA_TRY(cudaMemcpyAsync(parts.data(), s->loss_part, sizeof(float) * lb, cudaMemcpyDeviceToHost, s->stream));
        WC_CUDA_TRY(cudaStreamSynchronize(s->stream));
        double a = 0.0;
        for (float p : parts) a += p;
        *loss_host = (float)(a / ((double)rows * nout));
    }
    return WC_OK;
}

void init_params(wc_local* s, std::vector<float>& host) {
    host.assign(NPARAMS, 0.f);
    uint64_t st = 0x5EEDull * (s->cfg.seed + 1ull);
    auto uni = [&]() { return (float)((double)(splitmix64(st) >> 11) * (1.0 / 9007199254740992.0)) * 2.f - 1.f; };
    auto fill = [&](size_t off, uint32_t kin, uint32_t nout, uint32_t kin_used) {
        const float bound = std::sqrt(6.f / (float)(kin_used + nout));
        for (uint32_t k = 0; k < kin; ++k)
            for (uint32_t o = 0; o < nout; ++o) host[off + (size_t)k * nout + o] = k < kin_used ? bound * uni() : 0.f;
    };
    fill(OFF_W1, IN, HID, IN_USED);
    fill(OFF_W2, HID, HID, HID);
    fill(OFF_W3, HID, OUT, HID);
    for (uint32_t o = 0; o < OUT; ++o) host[OFF_W3 + o] *= 1.f;  // plain Glorot everywhere
    // the last layer starts small: the network starts close to the stale acceleration
    for (size_t i = 0; i < (size_t)HID * OUT; ++i) host[OFF_W3 + i] *= 0.1f;
}

wc_status ensure_roll(wc_local* s, uint32_t n) {
    if (n <= s->cap_roll) return WC_OK;
    dfree(s->change);
    dfree(s->mean_part);
    dfree(s->mean);
    dfree(s->judge_part);
    for (int q = 0; q < 2; ++q) {
        dfree(s->save_pos[q]);
        dfree(s->save_vel[q]);
        dfree(s->save_ids[q]);
    }
    s->cap_roll = 0;
    WC_TRY(dalloc(&s->change, (size_t)n * CHANGE_LD));
    if (!s->mean_part) WC_TRY(dalloc(&s->mean_part, (size_t)s->sms * MLP_CTAS_PER_SM * OUT));
    if (!s->mean) WC_TRY(dalloc(&s->mean, OUT));
    WC_TRY(dalloc(&s->judge_part, blocks_for(n, 32)));
    for (int q = 0; q < 2; ++q) {
        WC_TRY(dalloc(&s->save_pos[q], n));
        WC_TRY(dalloc(&s->save_vel[q], n));
        WC_TRY(dalloc(&s->save_ids[q], n));
    }
    s->cap_roll = n;
    return WC_OK;
}

}  // namespace

// ---- C ABI ------------------------------------------------------------------------------------------

extern "C" {

WC_API void wc_local_config_default(wc_local_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof *c);
    c->ages = 3;
    c->seed = 1;
    c->accel_scale = 10.0f;
    c->velocity_scale = 1.0f;
    c->capacity = 1ull << 24;
}

WC_API wc_status wc_local_create(const wc_local_config* c, wc_local** out) {
    clear_error();
    WC_NVTX("wc_local_create");
    if (!c || !out) return fail(WC_ERR_INVALID_ARG, "null argument");
    *out = nullptr;
    if (c->ages < 1 || c->ages > MAX_AGES) return fail(WC_ERR_INVALID_ARG, "ages must be in 1..%u", MAX_AGES);
    if (!(c->accel_scale > 0.f) || !(c->velocity_scale > 0.f)) return fail(WC_ERR_INVALID_ARG, "scales must be > 0");
    if (c->capacity == 0 || c->capacity > (1ull << 31)) return fail(WC_ERR_INVALID_ARG, "capacity must be in 1..2^31");
    wc_local* s = new (std::nothrow) wc_local();
    if (!s) return fail(WC_ERR_OOM, "host allocation failed");
    s->cfg = *c;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, dev);
    if (s->sms <= 0) s->sms = 1;
    wc_status st = WC_OK;
    if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess)
        st = fail(WC_ERR_CUDA, "stream creation failed");
    if (st == WC_OK) st = dalloc(&s->w, NPARAMS);
    if (st == WC_OK) st = dalloc(&s->g, NPARAMS);
    if (st == WC_OK) st = dalloc(&s->m, NPARAMS);
    if (st == WC_OK) st = dalloc(&s->v, NPARAMS);
    if (st == WC_OK) st = dalloc(&s->wb, NBF16);
    if (st == WC_OK) st = dalloc(&s->d_err, 1);
    if (st == WC_OK && cudaMallocHost(reinterpret_cast<void**>(&s->h_err), sizeof(uint32_t)) != cudaSuccess)
        st = fail(WC_ERR_OOM, "pinned host allocation failed");
    if (st == WC_OK && cudaMallocHost(reinterpret_cast<void**>(&s->h_judge), sizeof(double)) != cudaSuccess)
        st = fail(WC_ERR_OOM, "pinned host allocation failed");
    if (st == WC_OK) st = dalloc(&s->judge_out, 1);
    if (st == WC_OK) {
        std::vector<float> host;
        init_params(s, host);
        *s->h_err = 0;
        if (cudaMemcpyAsync(s->w, host.data(), sizeof(float) * NPARAMS, cudaMemcpyHostToDevice, s->stream) !=
                cudaSuccess ||
            cudaMemsetAsync(s->m, 0, sizeof(float) * NPARAMS, s->stream) != cudaSuccess ||
            cudaMemsetAsync(s->v, 0, sizeof(float) * NPARAMS, s->stream) != cudaSuccess ||
            cudaMemsetAsync(s->d_err, 0, sizeof(uint32_t), s->stream) != cudaSuccess ||
            cudaStreamSynchronize(s->stream) != cudaSuccess)
            st = fail(WC_ERR_CUDA, "parameter upload failed");
    }
    if (st != WC_OK) {
        free_local(s);
        delete s;
        return st;
    }
    *out = s;
    return WC_OK;
}

WC_API void wc_local_destroy(wc_local* s) {
    if (!s) return;
    if (s->stream) cudaStreamSynchronize(s->stream);
    free_local(s);
    delete s;
}

WC_API uint64_t wc_local_num_params(const wc_local* s) { return s ? NPARAMS : 0; }

WC_API wc_status wc_local_get_params(wc_local* s, float* out, uint64_t count) {
    clear_error();
    if (!s || !out || count != NPARAMS) return fail(WC_ERR_INVALID_ARG, "expected %zu parameters", NPARAMS);
    WC_CUDA_TRY(cudaMemcpyAsync(out, s->w, sizeof(float) * NPARAMS, cudaMemcpyDeviceToHost, s->stream));
    WC_CUDA_TRY(cudaStreamSynchronize(s->stream));
    return WC_OK;
}

WC_API wc_status wc_local_set_params(wc_local* s, const float* in, uint64_t count) {
    clear_error();
    if (!s || !in || count != NPARAMS) return fail(WC_ERR_INVALID_ARG, "expected %zu parameters", NPARAMS);
    WC_CUDA_TRY(cudaMemcpyAsync(s->w, in, sizeof(float) * NPARAMS, cudaMemcpyHostToDevice, s->stream));
    WC_CUDA_TRY(cudaMemsetAsync(s->m, 0, sizeof(float) * NPARAMS, s->stream));
    WC_CUDA_TRY(cudaMemsetAsync(s->v, 0, sizeof(float) * NPARAMS, s->stream));
    WC_CUDA_TRY(cudaStreamSynchronize(s->stream));
    s->adam_step = 0;
    s->cast_dirty = true;
    return WC_OK;
}

WC_API wc_status wc_local_record_fluid(wc_local* s, wc_fluid* f, float dt, uint32_t cycles, int held_out) {
    clear_error();
    WC_NVTX("wc_local_record_fluid");
    if (!s || !f) return fail(WC_ERR_INVALID_ARG, "null argument");
    if (!(dt > 0.f)) return fail(WC_ERR_INVALID_ARG, "dt must be > 0");
    WC_TRY(fluid_check(f));
    return record(s, fluid_target(f), dt, cycles, held_out ? 1 : 0);
}

WC_API wc_status wc_local_record_batch(wc_local* s, wc_batch* b, float dt, uint32_t cycles, int held_out) {
    clear_error();
    WC_NVTX("wc_local_record_batch");
    if (!s || !b) return fail(WC_ERR_INVALID_ARG, "null argument");
    if (!(dt > 0.f)) return fail(WC_ERR_INVALID_ARG, "dt must be > 0");
    WC_TRY(batch_check(b));
    return record(s, batch_target(b), dt, cycles, held_out ? 1 : 0);
}

WC_API uint64_t wc_local_num_samples(const wc_local* s, int held_out) { return s ? s->count[held_out ? 1 : 0] : 0; }

WC_API wc_status wc_local_clear_samples(wc_local* s) {
    clear_error();
    if (!s) return fail(WC_ERR_INVALID_ARG, "null argument");
    s->count[0] = s->count[1] = 0;
    return WC_OK;
}

WC_API wc_status wc_local_train(wc_local* s, uint32_t steps, uint32_t rows, float lr, float* loss) {
    clear_error();
    WC_NVTX("wc_local_train");
    if (!s) return fail(WC_ERR_INVALID_ARG, "null argument");
    if (rows == 0 || rows % 8) return fail(WC_ERR_INVALID_ARG, "rows must be a positive multiple of 8");
    if (s->count[0] == 0) return fail(WC_ERR_STATE, "no training samples (wc_local_record_*)");
    if (!(lr > 0.f)) return fail(WC_ERR_INVALID_ARG, "lr must be > 0");
    WC_TRY(ensure_train(s, rows));
    for (uint32_t k = 0; k < steps; ++k) {
        const uint64_t seed = 0xA5A5ull + 0x100000001B3ull * (uint64_t)(s->adam_step + 1);
        WC_TRY(train_step(s, rows, seed, nullptr, lr, loss ? loss + k : nullptr));
    }
    return read_err(s);
}

WC_API wc_status wc_local_gradients(wc_local* s, const uint32_t* rows_idx, uint32_t rows, float* grads, float* loss) {
    clear_error();
    if (!s || !rows_idx || !grads || !loss) return fail(WC_ERR_INVALID_ARG, "null argument");
    if (rows == 0 || rows % 8) return fail(WC_ERR_INVALID_ARG, "rows must be a positive multiple of 8");
    if (s->count[0] == 0) return fail(WC_ERR_STATE, "no training samples (wc_local_record_*)");
    WC_TRY(ensure_train(s, rows));
    uint32_t* d_idx = nullptr;
    WC_TRY(dalloc(&d_idx, rows));
    wc_status st = WC_OK;
    if (cudaMemcpyAsync(d_idx, rows_idx, sizeof(uint32_t) * rows, cudaMemcpyHostToDevice, s->stream) != cudaSuccess)
        st = fail(WC_ERR_CUDA, "index upload failed");
    if (st == WC_OK) st = train_step(s, rows, 0, d_idx, 0.f, loss);
    if (st == WC_OK &&
        (cudaMemcpyAsync(grads, s->g, sizeof(float) * NPARAMS, cudaMemcpyDeviceToHost, s->stream) != cudaSuccess ||
         cudaStreamSynchronize(s->stream) != cudaSuccess))
        st = fail(WC_ERR_CUDA, "gradient copy failed");
    cudaFree(d_idx);
    if (st != WC_OK) return st;
    return read_err(s);
}

WC_API wc_status wc_local_get_samples(wc_local* s, int held_out, uint64_t first, uint64_t count, float* inputs,
                                      float* targets) {
    clear_error();
    if (!s) return fail(WC_ERR_INVALID_ARG, "null argument");
    const int set = held_out ? 1 : 0;
    if (first + count > s->count[set]) return fail(WC_ERR_INVALID_ARG, "samples out of range");
    if (!count) return WC_OK;
    if (inputs) {
        std::vector<__nv_bfloat16> h((size_t)count * IN);
        WC_CUDA_TRY(cudaMemcpyAsync(h.data(), s->xs[set] + first * IN, sizeof(__nv_bfloat16) * h.size(),
                                    cudaMemcpyDeviceToHost, s->stream));
        WC_CUDA_TRY(cudaStreamSynchronize(s->stream));
        for (size_t i = 0; i < h.size(); ++i) inputs[i] = __bfloat162float(h[i]);
    }
    if (targets) {
        WC_CUDA_TRY(cudaMemcpyAsync(targets, s->ys[set] + first * YW, sizeof(float) * (size_t)count * YW,
                                    cudaMemcpyDeviceToHost, s->stream));
        WC_CUDA_TRY(cudaStreamSynchronize(s->stream));
    }
    return WC_OK;
}

WC_API wc_status wc_local_evaluate(wc_local* s, int held_out, float* err_net, float* err_stale, float* err_taylor) {
    clear_error();
    if (!s || !err_net || !err_stale) return fail(WC_ERR_INVALID_ARG, "null argument");
    const int set = held_out ? 1 : 0;
    const uint64_t rows = s->count[set];
    if (!rows) return fail(WC_ERR_STATE, "no samples in that set");
    if (rows > 0xFFFFFFFFull) return fail(WC_ERR_INVALID_ARG, "too many samples");
    cast(s);
    float* pred = nullptr;
    double* part = nullptr;
    const uint32_t blocks = blocks_for(rows, 128);
    WC_TRY(dalloc(&pred, rows * OUT));
    wc_status st = dalloc(&part, (size_t)blocks * EVAL_SUMS * MAX_AGES);
    if (st == WC_OK) {
        mlp_kernel<false, false><<<mlp_grid(s, (uint32_t)rows), MLP_THREADS, 0, s->stream>>>(
            (uint32_t)rows, InputSrc{}, s->xs[set], weights(s), pred, OUT, OUT, 1.0f, s->d_err);
        eval_kernel<<<blocks, 128, 0, s->stream>>>(rows, s->cfg.ages, s->xs[set], s->ys[set], pred, part);
        std::vector<double> h((size_t)blocks * EVAL_SUMS * MAX_AGES);
        if (cudaMemcpyAsync(h.data(), part, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, s->stream) !=
                cudaSuccess ||
            cudaStreamSynchronize(s->stream) != cudaSuccess)
            st = fail(WC_ERR_CUDA, "evaluation copy failed");
        if (st == WC_OK) {
            for (uint32_t g = 0; g < s->cfg.ages; ++g) {
                double sum[EVAL_SUMS] = {};
                for (uint32_t b = 0; b < blocks; ++b)
                    for (uint32_t q = 0; q < EVAL_SUMS; ++q) sum[q] += h[((size_t)b * MAX_AGES + g) * EVAL_SUMS + q];
                const double t = sum[3];
                err_net[g] = t > 0 ? (float)std::sqrt(sum[0] / t) : 0.f;
                err_stale[g] = t > 0 ? (float)std::sqrt(sum[1] / t) : 0.f;
                if (err_taylor) err_taylor[g] = t > 0 ? (float)std::sqrt(sum[2] / t) : 0.f;
            }
        }
    }
    cudaFree(pred);
    if (part) cudaFree(part);
    if (st != WC_OK) return st;
    return read_err(s);
}

WC_API wc_status wc_local_predict(wc_local* s, wc_fluid* f, float dt, float* inputs, float* outputs) {
    clear_error();
    if (!s || !f) return fail(WC_ERR_INVALID_ARG, "null argument");
    StepTarget t = fluid_target(f);
    const uint32_t n = t.d->n;
    WC_TRY(ensure_n(s, n));
    WC_TRY(ensure_roll(s, n));
    const bool had_accel = t.d->accel != nullptr;
    if (!had_accel) WC_TRY(wc_fluid_set_recording(f, 1));
    t = fluid_target(f);
    // the judge step's passes on a copy of the state: the fluid does not advance
    WC_CUDA_TRY(cudaMemcpyAsync(s->save_pos[0], t.d->pos_a, sizeof(float4) * n, cudaMemcpyDeviceToDevice, t.stream));
    WC_CUDA_TRY(cudaMemcpyAsync(s->save_vel[0], t.d->vel_a, sizeof(float4) * n, cudaMemcpyDeviceToDevice, t.stream));
    if (t.d->ids_a)
        WC_CUDA_TRY(cudaMemcpyAsync(s->save_ids[0], t.d->ids_a, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, t.stream));
    enqueue_judge_step(s, t, dt, false);
    cudaEvent_t ev;
    WC_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaEventRecord(ev, t.stream);
    cudaStreamWaitEvent(s->stream, ev, 0);
    enqueue_predict(s, t, dt);
    cudaEventRecord(ev, s->stream);
    cudaStreamWaitEvent(t.stream, ev, 0);
    cudaEventDestroy(ev);
    wc_status st = WC_OK;
    if (inputs && n) {
        __nv_bfloat16* xb = s->x_id;  // [n x IN] in sorted order (no ids)
        const InputSrc src = input_src(s, t, dt);
        inputs_kernel<false><<<blocks_for(n, 128), 128, 0, t.stream>>>(n, src, nullptr, xb);
        std::vector<__nv_bfloat16> h((size_t)n * IN);
        if (cudaMemcpyAsync(h.data(), xb, sizeof(__nv_bfloat16) * h.size(), cudaMemcpyDeviceToHost, t.stream) !=
                cudaSuccess ||
            cudaStreamSynchronize(t.stream) != cudaSuccess)
            st = fail(WC_ERR_CUDA, "input copy failed");
        for (size_t i = 0; i < h.size() && st == WC_OK; ++i) inputs[i] = __bfloat162float(h[i]);
    }
    if (st == WC_OK && outputs && n)
        if (cudaMemcpyAsync(outputs, s->change, sizeof(float) * (size_t)n * 3u * s->cfg.ages, cudaMemcpyDeviceToHost,
                            t.stream) != cudaSuccess)
            st = fail(WC_ERR_CUDA, "output copy failed");
    WC_CUDA_TRY(cudaMemcpyAsync(t.d->pos_a, s->save_pos[0], sizeof(float4) * n, cudaMemcpyDeviceToDevice, t.stream));
    WC_CUDA_TRY(cudaMemcpyAsync(t.d->vel_a, s->save_vel[0], sizeof(float4) * n, cudaMemcpyDeviceToDevice, t.stream));
    if (t.d->ids_a)
        WC_CUDA_TRY(cudaMemcpyAsync(t.d->ids_a, s->save_ids[0], sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, t.stream));
    WC_CUDA_TRY(cudaStreamSynchronize(t.stream));
    if (!had_accel) WC_TRY(wc_fluid_set_recording(f, 0));
    if (st != WC_OK) return st;
    WC_TRY(fluid_check(f));
    return read_err(s);
}

WC_API wc_status wc_local_rollout_mode(wc_local* s, wc_fluid* f, float dt, uint32_t nsteps, uint32_t ages,
                                       float tolerance, int mode, wc_rollout_stats* out) {
    clear_error();
    WC_NVTX("wc_local_rollout");
    if (!f || !out) return fail(WC_ERR_INVALID_ARG, "null argument");
    if (!(dt > 0.f)) return fail(WC_ERR_INVALID_ARG, "dt must be > 0");
    if (ages < 1 || ages > MAX_AGES) return fail(WC_ERR_INVALID_ARG, "ages must be in 1..%u", MAX_AGES);
    if (mode != WC_LOCAL_STALE && mode != WC_LOCAL_TAYLOR && mode != WC_LOCAL_NETWORK)
        return fail(WC_ERR_INVALID_ARG, "unknown rollout mode %d", mode);
    if (mode == WC_LOCAL_NETWORK && !s) return fail(WC_ERR_INVALID_ARG, "the network mode needs a network");
    if (mode == WC_LOCAL_NETWORK && ages > s->cfg.ages)
        return fail(WC_ERR_INVALID_ARG, "the network predicts %u ages", s->cfg.ages);
    wc_local* const net = mode == WC_LOCAL_NETWORK ? s : nullptr;
    const uint32_t taylor = mode != WC_LOCAL_STALE ? 1u : 0u;
    // the stale mode's judge steps need only the density rate (carried densities), not J
    const int level = mode == WC_LOCAL_STALE ? FEAT_RATE : FEAT_FULL;
    std::memset(out, 0, sizeof *out);
    // a rollout without a network handle still needs the judge's scratch: a private one
    wc_local* own = nullptr;
    if (!s) {
        wc_local_config c;
        wc_local_config_default(&c);
        c.capacity = 1;
        WC_TRY(wc_local_create(&c, &own));
    }
    wc_local* w = s ? s : own;
    StepTarget t = fluid_target(f);
    const uint32_t n = t.d->n;
    wc_status rc = ensure_n(w, n);
    if (rc == WC_OK) rc = ensure_roll(w, n);
    const bool had_accel = t.d->accel != nullptr;
    if (rc == WC_OK && !had_accel) rc = wc_fluid_set_recording(f, 1);
    if (rc == WC_OK) rc = fluid_check(f);
    double diag[6];
    if (rc == WC_OK) rc = fluid_diagnostics(f, diag);
    if (rc != WC_OK) {
        if (own) wc_local_destroy(own);
        return rc;
    }
    for (int q = 0; q < 6; ++q) out->diag_start[q] = diag[q];
    t = fluid_target(f);  // recording may have changed the buffers
    DevBuffers& d = *t.d;
    const bool ids = d.ids_a != nullptr;
    cudaEvent_t e0, e1, ej;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventCreateWithFlags(&ej, cudaEventDisableTiming);
    const auto w0 = std::chrono::steady_clock::now();
    cudaEventRecord(e0, t.stream);
    double err_sum = 0.0, err_max = 0.0;
    int cur = 0;  // save slot of this cycle's judge state
    bool have_prev = false;
    uint32_t done = 0;
    auto restore = [&](int slot) {
        cudaMemcpyAsync(d.pos_a, w->save_pos[slot], sizeof(float4) * n, cudaMemcpyDeviceToDevice, t.stream);
        cudaMemcpyAsync(d.vel_a, w->save_vel[slot], sizeof(float4) * n, cudaMemcpyDeviceToDevice, t.stream);
        if (ids) cudaMemcpyAsync(d.ids_a, w->save_ids[slot], sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, t.stream);
    };
    // The `count` skipped steps of the cycle whose judge state is in the state buffer, in one
    // kernel (the network's, or the stale acceleration's); the judge state goes to save slot `slot`.
    auto skip_steps = [&](uint32_t count, int slot) {
        if (!n || !count) return;
        SkipArgs k{d.pos_a, d.vel_a, d.accel, w->feat, w->save_pos[slot], w->save_vel[slot],
                   ids ? d.ids_a : nullptr, w->save_ids[slot], dt, count, taylor};
        if (net) {
            // the network's residuals and their mean over the particles, then the skipped steps
            cast(net);
            const InputSrc src = input_src(net, t, dt);
            const int grid = mlp_grid(net, n);
            mlp_kernel<true, false, true><<<grid, MLP_THREADS, 0, t.stream>>>(
                n, src, nullptr, weights(net), w->change, CHANGE_LD, CHANGE_LD, residual_scale(net, dt), net->d_err,
                w->mean_part);  // all CHANGE_LD columns (whole 16-byte stores); the skipped steps read 3 count
            output_mean_kernel<<<1, 32 * OUT, 0, t.stream>>>((uint32_t)grid, n, w->mean_part, w->mean);
            skip_cycle_kernel<false><<<blocks_for(n, 256), 256, 0, t.stream>>>(n, t.sc, BatchTables{}, k, w->change,
                                                                               CHANGE_LD, w->mean);
        } else {
            skip_cycle_kernel<false><<<blocks_for(n, 256), 256, 0, t.stream>>>(n, t.sc, BatchTables{}, k, nullptr, 0,
                                                                               nullptr);
        }
    };
    uint32_t last_skip = 0;  // skipped steps of the last cycle (judged at the end when > 0)
    while (rc == WC_OK && done < nsteps) {
        const uint32_t skip = std::min(ages, nsteps - done - 1u);
        enqueue_judge_step(w, t, dt, have_prev, level);
        if (have_prev) {
            cudaMemcpyAsync(w->h_judge, w->judge_out, sizeof(double), cudaMemcpyDeviceToHost, t.stream);
            cudaEventRecord(ej, t.stream);
        }
        skip_steps(skip, cur);  // speculative: replaced below when the judge reverts the last cycle
        if (have_prev) {
            if (cudaEventSynchronize(ej) != cudaSuccess) {
                rc = fail(WC_ERR_CUDA, "rollout: judge event failed");
                break;
            }
            const double err = n ? *w->h_judge / n : 0.0;
            err_sum += err;
            err_max = std::max(err_max, err);
            ++out->judged;
            if (!(err <= tolerance)) {
                // revert the previous cycle: its skipped steps again as plain SPH from the state
                // after its judge step, then this cycle's judge step and skipped steps again
                ++out->reverted;
                const int prev = cur ^ 1;
                restore(prev);
                for (uint32_t k = 0; k < last_skip && rc == WC_OK; ++k) rc = fluid_graph_step(f, dt);
                out->surrogate_steps -= last_skip;
                out->sph_steps += last_skip;
                enqueue_judge_step(w, t, dt, false, level);
                skip_steps(skip, cur);
            }
        }
        out->sph_steps += 1;
        out->surrogate_steps += skip;
        done += 1 + skip;
        have_prev = skip > 0;
        last_skip = skip;
        cur ^= 1;
    }
    if (rc == WC_OK && have_prev) {
        // the last cycle's skipped steps are judged too (a density pass on the final state)
        enqueue_closing_judge(w, t);
        cudaMemcpyAsync(w->h_judge, w->judge_out, sizeof(double), cudaMemcpyDeviceToHost, t.stream);
        if (cudaStreamSynchronize(t.stream) != cudaSuccess) {
            rc = fail(WC_ERR_CUDA, "rollout: closing judge failed");
        } else {
            const double err = n ? *w->h_judge / n : 0.0;
            err_sum += err;
            err_max = std::max(err_max, err);
            ++out->judged;
            if (!(err <= tolerance)) {
                ++out->reverted;
                restore(cur ^ 1);
                for (uint32_t k = 0; k < last_skip && rc == WC_OK; ++k) rc = fluid_graph_step(f, dt);
                out->surrogate_steps -= last_skip;
                out->sph_steps += last_skip;
            }
        }
    }
    for (uint32_t k = 0; k < done; ++k) fluid_count_step(f);
    cudaEventRecord(e1, t.stream);
    const cudaError_t ce = cudaStreamSynchronize(t.stream);
    const auto w1 = std::chrono::steady_clock::now();
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(ej);
    if (rc == WC_OK && ce != cudaSuccess) rc = fail(WC_ERR_CUDA, "rollout: %s", cudaGetErrorString(ce));
    if (rc == WC_OK) rc = fluid_check(f);
    if (rc == WC_OK) rc = read_err(w);
    if (!had_accel) {
        const wc_status r2 = wc_fluid_set_recording(f, 0);
        if (rc == WC_OK) rc = r2;
    }
    if (rc == WC_OK && fluid_diagnostics(f, diag) == WC_OK)
        for (int q = 0; q < 6; ++q) out->diag_end[q] = diag[q];
    if (own) wc_local_destroy(own);
    if (rc != WC_OK) return rc;
    out->steps = done;
    out->ms_device = ms;
    out->ms_wall = std::chrono::duration<double, std::milli>(w1 - w0).count();
    out->particle_steps_per_s = ms > 0 ? (double)n * done / (ms * 1e-3) : 0.0;
    out->mean_density_error = out->judged ? err_sum / out->judged : 0.0;
    out->max_density_error = err_max;
    return WC_OK;
}

WC_API wc_status wc_local_rollout(wc_local* s, wc_fluid* f, float dt, uint32_t nsteps, uint32_t ages, float tolerance,
                                  wc_rollout_stats* out) {
    return wc_local_rollout_mode(s, f, dt, nsteps, ages, tolerance, s ? WC_LOCAL_NETWORK : WC_LOCAL_STALE, out);
}

}  // extern "C"
