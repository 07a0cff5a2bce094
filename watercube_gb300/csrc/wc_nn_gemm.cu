// wc_nn_gemm.cu — BF16 tensor-core GEMM for the learned surrogate (sm_103a tcgen05 + TMEM).
//
//   C[m, n] = sum_k A[m, k] * B[k, n]        (BF16 operands, FP32 accumulation in TMEM)
//
// One CTA (4 warps) computes a 128 x 128 tile of C. Per 64-deep slice of K, all threads stage
// the A and B tiles into shared memory in the canonical no-swizzle K-major layout of the
// tensor-core descriptors (8-row x 16-byte core matrices; the next core matrix along K is 128 B
// away, the next 8-row group 1,024 B away), fence them into the async proxy, and one thread
// issues four tcgen05.mma (K = 16 each) into a 128-column FP32 accumulator in tensor memory and
// commits them to an mbarrier. The epilogue reads the accumulator with tcgen05.ld (warp w owns
// rows 32w..32w+31, one row per thread) and applies bias, row gathers, ReLU and the store.
//
// Operand sources (staging policies):
//   A row-major [m x k] (lda), optionally with a row index (gather) and a second source for
//     the columns at and after k_split (concatenation [X | Y]); or A transposed: A[i][kk] =
//     a[kk * lda + i] (the weight-gradient GEMM X^T dY).
//   B as B^T row-major [n x k] (ldb) (a weight matrix stored output-major), or B row-major
//     [k x n] (the upstream gradient dY in X^T dY, and W in dY W^T).
// Every wait on the mbarrier is bounded; a wait that runs out sets an error flag, and the
// kernel still releases its tensor memory before it returns.
//
// Two kernels: gemm_pipe_kernel (persistent, warp-specialised, an operand ring, B resident in
// shared memory when it fits, two accumulators, see below) for row-major operands without a
// split of K — the forward layers and the input gradients; gemm_kernel (one tile per CTA, two operand buffers) for the transposed
// weight-gradient operands and split-K.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "wc_internal.h"
#include "wc_nn.h"
#include "wc_util.h"

namespace wc {
namespace nn {
namespace {

constexpr int BM = 128, BN = 128, BK = 64;
constexpr int THREADS = 128;
constexpr uint32_t TMEM_COLS = 128;
constexpr uint32_t WAIT_LIMIT = 1u << 22;

// Instruction descriptor of tcgen05.mma kind::f16: FP32 accumulator (bits 4-5 = 1), BF16 A and
// B (bits 7-9 = 1, bits 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at bit 24.
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(BN >> 3) << 17) |
                           ((uint32_t)(BM >> 4) << 24);

// Two buffers of each operand tile: the threads stage slice k+1 into one while the tensor core
// still reads slice k from the other.
struct __align__(1024) Tiles {
    __nv_bfloat16 a[2][BM * BK];  // 2 x 16 KB
    __nv_bfloat16 b[2][BN * BK];  // 2 x 16 KB
};

__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: start >> 4, LBO = 128 B (next core matrix along K),
// SBO = 1024 B (next 8-row group), version 1, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)(128u >> 4) << 16;
    d |= (uint64_t)(1024u >> 4) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Byte offset of element (r, k) of a 128 x 64 tile in the core-matrix layout.
__device__ __forceinline__ uint32_t tile_off(uint32_t r, uint32_t k) {
    return (((r >> 3) * 8u + (k >> 3)) << 7) + ((r & 7u) << 4) + ((k & 7u) << 1);
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

// Stage a 128 x 64 slice of an operand: rows [row0, row0 + 128) of the logical matrix, columns
// [k0, k0 + 64). T = transposed source (logical (r, k) = src[k * ld + r]).
struct OperandSrc {
    const __nv_bfloat16* p;   // primary source
    const __nv_bfloat16* p2;  // second source for columns >= k_split (row-major only), or null
    const uint32_t* rows;     // row gather (row-major only), or null
    uint32_t ld, ld2, k_split;
    uint32_t nrows, ncols;    // logical extent
    int transposed;
};

__device__ __forceinline__ void stage(const OperandSrc& s, __nv_bfloat16* tile, uint32_t row0, uint32_t k0) {
    unsigned char* base = reinterpret_cast<unsigned char*>(tile);
    if (!s.transposed) {
        // 1,024 chunks of 8 elements (16 B); chunk id -> (row r, k-group g).
        for (uint32_t id = threadIdx.x; id < (uint32_t)(BM * BK / 8); id += THREADS) {
            const uint32_t r = id >> 3, g = id & 7u;
            const uint32_t row = row0 + r, col = k0 + 8u * g;
            uint4 v = make_uint4(0u, 0u, 0u, 0u);
            if (row < s.nrows && col < s.ncols) {
                const uint32_t src_row = s.rows ? __ldg(s.rows + row) : row;
                const __nv_bfloat16* src;
                if (s.p2 && col >= s.k_split)
                    src = s.p2 + (size_t)src_row * s.ld2 + (col - s.k_split);
                else
                    src = s.p + (size_t)src_row * s.ld + col;
                v = __ldg(reinterpret_cast<const uint4*>(src));
            }
            *reinterpret_cast<uint4*>(base + tile_off(r, 8u * g)) = v;
        }
    } else {
        // 128 blocks of 8 logical rows x 8 k: eight 16-byte loads (8 rows at one k each),
        // transposed in registers with byte permutes into eight 16-byte core-matrix rows.
        for (uint32_t b = threadIdx.x; b < (uint32_t)((BM / 8) * (BK / 8)); b += THREADS) {
            const uint32_t kg = b >> 4, rg = b & 15u;
            const uint32_t r = row0 + 8u * rg;
            uint4 v[8];
#pragma unroll
            for (uint32_t e = 0; e < 8; ++e) {
                const uint32_t kk = k0 + 8u * kg + e;
                v[e] = make_uint4(0u, 0u, 0u, 0u);
                if (kk < s.ncols && r < s.nrows) v[e] = __ldg(reinterpret_cast<const uint4*>(s.p + (size_t)kk * s.ld + r));
            }
#pragma unroll
            for (uint32_t j = 0; j < 8; ++j) {
                // row 8 rg + j: element e of the output row is element j of v[e]
                const uint32_t sel = (j & 1u) ? 0x7632u : 0x5410u;
                const uint32_t q = j >> 1;
                auto word = [&](const uint4& x) { return q == 0 ? x.x : q == 1 ? x.y : q == 2 ? x.z : x.w; };
                uint4 w;
                w.x = __byte_perm(word(v[0]), word(v[1]), sel);
                w.y = __byte_perm(word(v[2]), word(v[3]), sel);
                w.z = __byte_perm(word(v[4]), word(v[5]), sel);
                w.w = __byte_perm(word(v[6]), word(v[7]), sel);
                *reinterpret_cast<uint4*>(base + tile_off(8u * rg + j, 8u * kg)) = w;
            }
        }
    }
}

// The row-major staging as asynchronous copies (cp.async, 16 bytes each, zero-filled outside the
// matrix): no registers, and the copies of the next slice run while the tensor core works.
__device__ __forceinline__ void stage_async(const OperandSrc& s, __nv_bfloat16* tile, uint32_t row0, uint32_t k0) {
    const uint32_t base = smem_addr(tile);
#pragma unroll 4
    for (uint32_t id = threadIdx.x; id < (uint32_t)(BM * BK / 8); id += THREADS) {
        const uint32_t r = id >> 3, g = id & 7u;
        const uint32_t row = row0 + r, col = k0 + 8u * g;
        const __nv_bfloat16* src = s.p;  // nothing is read when bytes = 0
        uint32_t bytes = 0;
        if (row < s.nrows && col < s.ncols) {
            const uint32_t src_row = s.rows ? __ldg(s.rows + row) : row;
            if (s.p2 && col >= s.k_split)
                src = s.p2 + (size_t)src_row * s.ld2 + (col - s.k_split);
            else
                src = s.p + (size_t)src_row * s.ld + col;
            bytes = 16;
        }
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(base + tile_off(r, 8u * g)), "l"(src),
                     "r"(bytes)
                     : "memory");
    }
}

// x[0..ncols) += r[0..ncols) (bf16): 16-byte loads when the row segment is whole and aligned.
__device__ __forceinline__ void add_row(float x[32], const __nv_bfloat16* r, uint32_t ncols) {
    if (ncols == 32u && (reinterpret_cast<uintptr_t>(r) & 15u) == 0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint4 v = __ldg(reinterpret_cast<const uint4*>(r) + q);
            const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&v);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float2 f = __bfloat1622float2(h[k]);
                x[8 * q + 2 * k] += f.x;
                x[8 * q + 2 * k + 1] += f.y;
            }
        }
    } else {
#pragma unroll
        for (int j = 0; j < 32; ++j)
            if ((uint32_t)j < ncols) x[j] += __bfloat162float(r[j]);
    }
}

// Bias, gathered row adds, ReLU and the stores of 32 accumulator columns of one row:
// x[0..ncols) belong to output columns col0 ..; kz: the split of the K range (partial outputs
// split_stride apart).
__device__ __forceinline__ void epilogue_store(const GemmArgs& g, float x[32], uint32_t row, uint32_t col0,
                                               uint32_t ncols, uint32_t kz) {
    if (g.bias) {
#pragma unroll
        for (int j = 0; j < 32; ++j)
            if ((uint32_t)j < ncols) x[j] += __ldg(g.bias + col0 + j);
    }
    if (g.add1) add_row(x, g.add1 + (size_t)__ldg(g.add1_idx + row) * g.ld_add + col0, ncols);
    if (g.add2) add_row(x, g.add2 + (size_t)__ldg(g.add2_idx + row) * g.ld_add + col0, ncols);
    if (g.relu) {
#pragma unroll
        for (int j = 0; j < 32; ++j) x[j] = fmaxf(x[j], 0.f);
    }
    // Stores: 16-byte vectors for whole aligned segments, otherwise element by element with
    // constant indices (the accumulator stays in registers either way).
    if (g.c_f32) {
        float* out = g.c_f32 + (size_t)kz * g.split_stride + (size_t)row * g.ldc + col0;
        if (ncols == 32 && ((reinterpret_cast<uintptr_t>(out) & 15u) == 0)) {
#pragma unroll
            for (int j = 0; j < 32; j += 4) {
                float4* o = reinterpret_cast<float4*>(out + j);
                float4 v = make_float4(x[j], x[j + 1], x[j + 2], x[j + 3]);
                if (g.accumulate) {
                    const float4 c = *o;
                    v.x += c.x;
                    v.y += c.y;
                    v.z += c.z;
                    v.w += c.w;
                }
                *o = v;
            }
        } else {
#pragma unroll
            for (int j = 0; j < 32; ++j)
                if ((uint32_t)j < ncols) out[j] = g.accumulate ? out[j] + x[j] : x[j];
        }
    }
    if (g.c_bf16) {
        __nv_bfloat16* out = g.c_bf16 + (size_t)row * g.ldc + col0;
        if (ncols == 32 && ((reinterpret_cast<uintptr_t>(out) & 15u) == 0)) {
#pragma unroll
            for (int j = 0; j < 32; j += 8) {
                __nv_bfloat162 q0 = __floats2bfloat162_rn(x[j], x[j + 1]);
                __nv_bfloat162 q1 = __floats2bfloat162_rn(x[j + 2], x[j + 3]);
                __nv_bfloat162 q2 = __floats2bfloat162_rn(x[j + 4], x[j + 5]);
                __nv_bfloat162 q3 = __floats2bfloat162_rn(x[j + 6], x[j + 7]);
                uint4 w;
                w.x = *reinterpret_cast<uint32_t*>(&q0);
                w.y = *reinterpret_cast<uint32_t*>(&q1);
                w.z = *reinterpret_cast<uint32_t*>(&q2);
                w.w = *reinterpret_cast<uint32_t*>(&q3);
                *reinterpret_cast<uint4*>(out + j) = w;
            }
        } else {
#pragma unroll
            for (int j = 0; j < 32; ++j)
                if ((uint32_t)j < ncols) out[j] = __float2bfloat16_rn(x[j]);
        }
    }

}

__global__ void __launch_bounds__(THREADS) gemm_kernel(const GemmArgs g, uint32_t* err) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    Tiles& t = *reinterpret_cast<Tiles*>(smem_raw);
    __shared__ uint64_t mbar[2];  // MMA completion per operand buffer
    __shared__ uint32_t tmem_slot;
    __shared__ int s_failed;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    const uint32_t kz = blockIdx.z;  // split of the K range (weight gradients)
    const uint32_t k_begin = kz * g.k_chunk;
    const uint32_t k_end = min(g.k, k_begin + g.k_chunk);

    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&mbar[0])));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&mbar[1])));
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

    OperandSrc A{g.a, g.a2, g.a_rows, g.lda, g.lda2, g.k_split, g.m, g.k, g.a_transposed};
    // B is staged as B^T (rows = output columns n, columns = k).
    OperandSrc B{g.b, nullptr, nullptr, g.ldb, 0u, 0u, g.n, g.k, g.b_rowmajor};

    uint32_t phase[2] = {0u, 0u};
    bool pending[2] = {false, false};  // an MMA batch reading this buffer may still run
    bool ok = true;
    uint32_t issued = 0;
    int last = -1;
    // Both operands row-major: asynchronous copies, one slice ahead. Otherwise the threads stage
    // through registers (the transposed forms), still into the buffer the tensor core is not
    // reading.
    const bool async = !A.transposed && !B.transposed;
    if (async && k_begin < k_end) {
        stage_async(A, t.a[0], m0, k_begin);
        stage_async(B, t.b[0], n0, k_begin);
        asm volatile("cp.async.commit_group;" ::: "memory");
    }
    for (uint32_t k0 = k_begin; k0 < k_end; k0 += BK) {
        const int buf = (int)(issued & 1u);
        if (async) {
            const uint32_t kn = k0 + BK;
            if (kn < k_end) {
                const int nb = buf ^ 1;
                if (pending[nb]) {
                    // the batch that read buffer nb (one slice back) must finish before the rewrite
                    if (!mbar_wait(smem_addr(&mbar[nb]), phase[nb])) ok = false;
                    phase[nb] ^= 1u;
                    pending[nb] = false;
                }
                stage_async(A, t.a[nb], m0, kn);
                stage_async(B, t.b[nb], n0, kn);
                asm volatile("cp.async.commit_group;" ::: "memory");
                asm volatile("cp.async.wait_group 1;" ::: "memory");  // this slice's copies are done
            } else {
                asm volatile("cp.async.wait_group 0;" ::: "memory");
            }
        } else {
            if (pending[buf]) {
                // The batch two slices back read this buffer: it must finish before the rewrite.
                if (!mbar_wait(smem_addr(&mbar[buf]), phase[buf])) ok = false;
                phase[buf] ^= 1u;
                pending[buf] = false;
            }
            stage(A, t.a[buf], m0, k0);
            stage(B, t.b[buf], n0, k0);
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (threadIdx.x == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a_base = smem_addr(t.a[buf]), b_base = smem_addr(t.b[buf]);
#pragma unroll
            for (uint32_t j = 0; j < BK / 16; ++j) {
                const uint64_t ad = smem_desc(a_base + 256u * j);
                const uint64_t bd = smem_desc(b_base + 256u * j);
                const uint32_t acc = (issued > 0 || j > 0) ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(IDESC), "r"(acc));
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_addr(&mbar[buf]))
                         : "memory");
        }
        pending[buf] = true;
        last = buf;
        ++issued;
    }
    // The last commit covers every MMA issued before it; the other buffer's arrival needs no wait.
    if (last >= 0) {
        if (!mbar_wait(smem_addr(&mbar[last]), phase[last])) ok = false;
    }
    if (!ok) atomicOr(&s_failed, 1);
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    __syncthreads();
    const bool failed = s_failed != 0;
    if (failed && threadIdx.x == 0 && err) atomicOr(err, DEVERR_MMA_TIMEOUT);

    // Epilogue: thread owns row m0 + 32 warp + lane; columns in chunks of 32.
    const uint32_t row = m0 + 32u * warp + lane;
    const bool row_ok = row < g.m && !failed;
    for (uint32_t c0 = 0; c0 < BN; c0 += 32) {
        uint32_t v[32];
        const uint32_t taddr = tmem + ((32u * warp) << 16) + c0;
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
            "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
              "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
              "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
              "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
            : "r"(taddr));
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (!row_ok || n0 + c0 >= g.n) continue;
        float x[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) x[j] = issued ? __uint_as_float(v[j]) : 0.f;
        epilogue_store(g, x, row, n0 + c0, min(32u, g.n - (n0 + c0)), kz);
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
    }
}

// ---- persistent, warp-specialised kernel (row-major A with gather / concatenation, B^T) --------
//
// Grid: one CTA per SM, looping over output tiles. Warps 0..3 (the producers) copy operand
// slices with cp.async into a ring of shared-memory slots, one commit group per ring step, and
// keep LAG groups in flight: after committing a group a thread waits until only the LAG newest
// are pending, fences the older ones into the async proxy and arrives on their `full` barriers.
// With B resident (RB: n <= 128 and k <= 384) the producers first copy the whole B^T tile once
// (barrier `b_full`) and the ring carries A slices only (6 slots, 4 in flight); otherwise each
// slot holds an A and a B slice (4 slots, 2 in flight). Warp 4 (lane 0) waits for `full`, issues
// the slice's four MMAs into one of two 128-column accumulators in tensor memory and commits them
// to the slot's `empty` barrier (the slot may be refilled) and, after a tile's last slice, to the
// accumulator's `acc_full` barrier. Warps 5..12 wait for `acc_full`, read 32 accumulator rows x 64
// columns each (warp w reads lanes 32 (w % 4) ..), apply the epilogue and arrive on `acc_empty`. So
// the copies of the next slices, the MMAs of one tile and the epilogue of the previous tile
// overlap. Every wait is bounded; a wait that runs out stops the CTA's loops
// (DEVERR_MMA_TIMEOUT) and the CTA still frees its tensor memory.
constexpr int PIPE_PRODUCERS = 4;  // warps 0..3 copy, warp 4 issues the MMAs, warps 5..12 drain
constexpr int PIPE_EPILOGUE = 8;   // two warps per 32-lane quarter of the accumulator, 64 columns each
constexpr int PIPE_THREADS = 32 * (PIPE_PRODUCERS + 1 + PIPE_EPILOGUE);
constexpr uint32_t PIPE_TMEM_COLS = 256;
constexpr uint32_t TILE_BYTES = BM * BK * 2;  // one 128 x 64 BF16 operand slice, 16 KB
// Resident B (RB): the whole B^T tile [128 x k] stays in shared memory, loaded once per CTA,
// and the ring carries A slices only. For n <= 128 (one column of tiles) and k <= 64 RB_MAX_SLICES.
constexpr uint32_t RB_MAX_SLICES = 6;
template <bool RB>
struct PipeShape {
    static constexpr int STAGES = RB ? 6 : 4;  // ring slots
    static constexpr int LAG = STAGES - 2;     // copy groups a producer keeps in flight
};

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}\n" ::"r"(smem_addr(bar)) : "memory");
}

// A producer thread's share of one slice: 16-byte copies (PIPE_PRODUCERS warps), zero-filled
// outside the matrix.
__device__ __forceinline__ void pipe_stage_copy(const OperandSrc& s, __nv_bfloat16* tile, uint32_t row0, uint32_t k0,
                                                uint32_t ptid) {
    const uint32_t base = smem_addr(tile);
#pragma unroll 4
    for (uint32_t id = ptid; id < (uint32_t)(BM * BK / 8); id += 32u * PIPE_PRODUCERS) {
        const uint32_t r = id >> 3, g = id & 7u;
        const uint32_t row = row0 + r, col = k0 + 8u * g;
        const __nv_bfloat16* src = s.p;
        uint32_t bytes = 0;
        if (row < s.nrows && col < s.ncols) {
            const uint32_t src_row = s.rows ? __ldg(s.rows + row) : row;
            if (s.p2 && col >= s.k_split)
                src = s.p2 + (size_t)src_row * s.ld2 + (col - s.k_split);
            else
                src = s.p + (size_t)src_row * s.ld + col;
            bytes = 16;
        }
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(base + tile_off(r, 8u * g)), "l"(src),
                     "r"(bytes)
                     : "memory");
    }
}

// The epilogue warps of the persistent kernels: for each of the CTA's tiles wait for its
// accumulator (acc_full[t & 1]), read 32 rows (lanes 32 quarter ..) x 64 columns (64 half ..)
// with tcgen05.ld, apply the epilogue, and hand the accumulator back (acc_empty). A wait that runs
// out sets `failed`.
__device__ __forceinline__ void drain_accumulators(const GemmArgs& g, uint32_t tmem, uint64_t* acc_full,
                                                   uint64_t* acc_empty, volatile int* failed, uint32_t ntiles,
                                                   uint32_t tiles_n, uint32_t nslices, uint32_t quarter,
                                                   uint32_t half, uint32_t lane) {
    uint32_t t = 0;
    for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++t) {
        const uint32_t b = t & 1u;
        bool ok = !*failed && mbar_wait(smem_addr(&acc_full[b]), (t >> 1) & 1u);
        ok = __all_sync(0xffffffffu, ok);
        if (!ok) {
            if (lane == 0) *failed = 1;
            break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t m0 = (tile / tiles_n) * BM, n0 = (tile % tiles_n) * BN;
        const uint32_t row = m0 + 32u * quarter + lane;
        const bool row_ok = row < g.m;
        for (uint32_t c0 = 64u * half; c0 < 64u * half + 64u; c0 += 32) {
            uint32_t v[32];
            const uint32_t taddr = tmem + ((32u * quarter) << 16) + b * (uint32_t)BN + c0;
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15]), "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]),
                  "=r"(v[22]), "=r"(v[23]), "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]),
                  "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
                : "r"(taddr));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (!row_ok || n0 + c0 >= g.n) continue;
            float x[32];
#pragma unroll
            for (int j = 0; j < 32; ++j) x[j] = nslices ? __uint_as_float(v[j]) : 0.f;
            epilogue_store(g, x, row, n0 + c0, min(32u, g.n - (n0 + c0)), 0u);
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncwarp();
        if (lane == 0) mbar_arrive(&acc_empty[b]);
    }
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t v[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
          "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]),
          "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
          "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr));
}

// The LayerNorm epilogue (GemmArgs::ln_gamma, n = 128, one column of tiles): the two warps that
// read the same 32 accumulator lanes (`quarter`) hold a row's 128 columns between them, 64 each
// (`half`). Each thread sums its 64 values, the pair exchanges the sums through shared memory at
// a named barrier of its 64 threads (ids 1 .. 4), then the squared deviations from the mean the
// same way, and each thread normalises, scales and shifts its own columns, adds the residual row
// and stores BF16. Both warps of a pair pass both barriers of every tile: whether each warp's
// accumulator wait succeeded is exchanged at the first barrier and the pair leaves together.
__device__ __forceinline__ void pair_sync(uint32_t quarter) {
    asm volatile("bar.sync %0, 64;" ::"r"(1u + quarter) : "memory");
}

__device__ __forceinline__ void drain_accumulators_ln(const GemmArgs& g, uint32_t tmem, uint64_t* acc_full,
                                                      uint64_t* acc_empty, volatile int* failed, uint32_t ntiles,
                                                      uint32_t nslices, uint32_t quarter, uint32_t half,
                                                      uint32_t lane, float (*xs)[2][32], float (*xv)[2][32],
                                                      int (*oks)[2]) {
    constexpr float LN_EPSILON = 1e-5f;
    const uint32_t col0 = 64u * half;
    // bias, gamma and beta four at a time when all three allow 16-byte loads (uniform branch)
    const bool vec = ((reinterpret_cast<uintptr_t>(g.ln_gamma) | reinterpret_cast<uintptr_t>(g.ln_beta) |
                       reinterpret_cast<uintptr_t>(g.bias)) & 15u) == 0;
    uint32_t t = 0;
    for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++t) {
        const uint32_t b = t & 1u;
        bool ok = !*failed && mbar_wait(smem_addr(&acc_full[b]), (t >> 1) & 1u);
        ok = __all_sync(0xffffffffu, ok);
        float x[64];
        if (ok) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t taddr = tmem + ((32u * quarter) << 16) + b * (uint32_t)BN + col0;
            uint32_t v[32];
            tmem_ld32(taddr, v);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int j = 0; j < 32; ++j) x[j] = nslices ? __uint_as_float(v[j]) : 0.f;
            tmem_ld32(taddr + 32u, v);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int j = 0; j < 32; ++j) x[32 + j] = nslices ? __uint_as_float(v[j]) : 0.f;
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(&acc_empty[b]);
        } else {
#pragma unroll
            for (int j = 0; j < 64; ++j) x[j] = 0.f;
        }
        if (g.bias) {
            if (vec) {
#pragma unroll
                for (int j = 0; j < 64; j += 4) {
                    const float4 bb = __ldg(reinterpret_cast<const float4*>(g.bias + col0 + j));
                    x[j] += bb.x;
                    x[j + 1] += bb.y;
                    x[j + 2] += bb.z;
                    x[j + 3] += bb.w;
                }
            } else {
#pragma unroll
                for (int j = 0; j < 64; ++j) x[j] += __ldg(g.bias + col0 + j);
            }
        }
        float sum = 0.f;
#pragma unroll
        for (int j = 0; j < 64; ++j) sum += x[j];
        xs[quarter][half][lane] = sum;
        if (lane == 0) oks[quarter][half] = ok ? 1 : 0;
        pair_sync(quarter);
        if (!(oks[quarter][0] && oks[quarter][1])) {
            if (lane == 0) *failed = 1;
            break;
        }
        const float mean = (xs[quarter][0][lane] + xs[quarter][1][lane]) * (1.f / 128.f);
        float sq = 0.f;
#pragma unroll
        for (int j = 0; j < 64; ++j) {
            x[j] -= mean;
            sq += x[j] * x[j];
        }
        xv[quarter][half][lane] = sq;
        pair_sync(quarter);
        const float var = (xv[quarter][0][lane] + xv[quarter][1][lane]) * (1.f / 128.f);
        const float rstd = rsqrtf(var + LN_EPSILON);
        const uint32_t row = tile * BM + 32u * quarter + lane;
        if (row >= g.m) continue;
        const __nv_bfloat16* res = g.ln_resid ? g.ln_resid + (size_t)row * 128u + col0 : nullptr;
        __nv_bfloat16* out = g.c_bf16 + (size_t)row * g.ldc + col0;
#pragma unroll
        for (int c = 0; c < 64; c += 8) {
            float gm[8], bt[8];
            if (vec) {
#pragma unroll
                for (int k = 0; k < 8; k += 4) {
                    const float4 g4 = __ldg(reinterpret_cast<const float4*>(g.ln_gamma + col0 + c + k));
                    const float4 b4 = __ldg(reinterpret_cast<const float4*>(g.ln_beta + col0 + c + k));
                    gm[k] = g4.x, gm[k + 1] = g4.y, gm[k + 2] = g4.z, gm[k + 3] = g4.w;
                    bt[k] = b4.x, bt[k + 1] = b4.y, bt[k + 2] = b4.z, bt[k + 3] = b4.w;
                }
            } else {
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    gm[k] = __ldg(g.ln_gamma + col0 + c + k);
                    bt[k] = __ldg(g.ln_beta + col0 + c + k);
                }
            }
            float o[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) o[k] = x[c + k] * rstd * gm[k] + bt[k];
            if (res) {
                const uint4 rv = __ldg(reinterpret_cast<const uint4*>(res + c));
                const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&rv);
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    const float2 f = __bfloat1622float2(h[k]);
                    o[2 * k] += f.x;
                    o[2 * k + 1] += f.y;
                }
            }
            uint4 w;
            __nv_bfloat162 q0 = __floats2bfloat162_rn(o[0], o[1]), q1 = __floats2bfloat162_rn(o[2], o[3]);
            __nv_bfloat162 q2 = __floats2bfloat162_rn(o[4], o[5]), q3 = __floats2bfloat162_rn(o[6], o[7]);
            w.x = *reinterpret_cast<uint32_t*>(&q0);
            w.y = *reinterpret_cast<uint32_t*>(&q1);
            w.z = *reinterpret_cast<uint32_t*>(&q2);
            w.w = *reinterpret_cast<uint32_t*>(&q3);
            *reinterpret_cast<uint4*>(out + c) = w;
        }
    }
}

template <bool RB>
__global__ void __launch_bounds__(PIPE_THREADS, 1) gemm_pipe_kernel(const GemmArgs g, uint32_t* err) {
    constexpr int STAGES = PipeShape<RB>::STAGES, LAG = PipeShape<RB>::LAG;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ uint64_t full[STAGES], empty[STAGES], acc_full[2], acc_empty[2], b_full;
    __shared__ uint32_t tmem_slot;
    __shared__ int s_failed;
    volatile int* failed = &s_failed;  // polled by all three roles
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t tiles_m = (g.m + BM - 1) / BM, tiles_n = (g.n + BN - 1) / BN;
    const uint32_t ntiles = tiles_m * tiles_n;
    const uint32_t nslices = (g.k + BK - 1) / BK;
    // RB: [B slices 0 .. nslices)[A ring]; otherwise the ring's slots hold an A and a B slice each
    unsigned char* const ring = smem_raw + (RB ? nslices * TILE_BYTES : 0u);
    auto a_slot = [&](uint32_t st) { return ring + st * (RB ? 1u : 2u) * TILE_BYTES; };
    auto b_slice = [&](uint32_t st, uint32_t sl) {
        return RB ? smem_raw + sl * TILE_BYTES : ring + (2u * st + 1u) * TILE_BYTES;
    };

    if (threadIdx.x == 0) {
        for (int q = 0; q < STAGES; ++q) {
            mbar_init(&full[q], 32 * PIPE_PRODUCERS);
            mbar_init(&empty[q], 1);
        }
        for (int q = 0; q < 2; ++q) {
            mbar_init(&acc_full[q], 1);
            mbar_init(&acc_empty[q], PIPE_EPILOGUE);  // one arrival per epilogue warp
        }
        mbar_init(&b_full, 32 * PIPE_PRODUCERS);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_failed = 0;
    }
    if (warp == PIPE_PRODUCERS) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_slot)),
                     "r"(PIPE_TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;
    const OperandSrc A{g.a, g.a2, g.a_rows, g.lda, g.lda2, g.k_split, g.m, g.k, 0};
    const OperandSrc B{g.b, nullptr, nullptr, g.ldb, 0u, 0u, g.n, g.k, 0};

    if (warp < PIPE_PRODUCERS) {
        // producers: copy groups in commit order (RB: group 0 is B, group 1 + i the A slice of
        // ring step i; otherwise group i is ring step i); a group is published (fenced, its
        // barrier arrived on) once LAG later groups have been committed, or at the end
        const uint32_t ptid = threadIdx.x;
        uint32_t it = 0, committed = 0, published = 0;
        auto publish_upto = [&](uint32_t upto) {
            for (; published < upto; ++published) {
                if (RB && published == 0)
                    mbar_arrive(&b_full);
                else
                    mbar_arrive(&full[(published - (RB ? 1u : 0u)) % STAGES]);
            }
        };
        if (RB) {
            for (uint32_t sl = 0; sl < nslices; ++sl)
                pipe_stage_copy(B, reinterpret_cast<__nv_bfloat16*>(b_slice(0, sl)), 0u, sl * BK, ptid);
            asm volatile("cp.async.commit_group;" ::: "memory");
            ++committed;
        }
        for (uint32_t tile = blockIdx.x; tile < ntiles && !*failed; tile += gridDim.x) {
            const uint32_t m0 = (tile / tiles_n) * BM, n0 = (tile % tiles_n) * BN;
            for (uint32_t sl = 0; sl < nslices; ++sl, ++it) {
                const uint32_t st = it % STAGES;
                if (it >= (uint32_t)STAGES && !mbar_wait(smem_addr(&empty[st]), ((it / STAGES) - 1u) & 1u)) {
                    *failed = 1;
                    break;
                }
                pipe_stage_copy(A, reinterpret_cast<__nv_bfloat16*>(a_slot(st)), m0, sl * BK, ptid);
                if (!RB) pipe_stage_copy(B, reinterpret_cast<__nv_bfloat16*>(b_slice(st, sl)), n0, sl * BK, ptid);
                asm volatile("cp.async.commit_group;" ::: "memory");
                ++committed;
                if (committed > (uint32_t)LAG) {
                    asm volatile("cp.async.wait_group %0;" ::"n"(LAG) : "memory");
                    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                    publish_upto(committed - LAG);
                }
            }
            if (*failed) break;
        }
        // the last groups
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        publish_upto(committed);
    } else if (warp == PIPE_PRODUCERS) {
        // MMA issue (one thread)
        if (lane == 0) {
            uint32_t it = 0, t = 0;
            if (RB && ntiles > blockIdx.x && !mbar_wait(smem_addr(&b_full), 0u)) *failed = 1;
            for (uint32_t tile = blockIdx.x; tile < ntiles && !*failed; tile += gridDim.x, ++t) {
                const uint32_t b = t & 1u;
                if (t >= 2 && !mbar_wait(smem_addr(&acc_empty[b]), ((t >> 1) - 1u) & 1u)) {
                    *failed = 1;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t acc_addr = tmem + b * (uint32_t)BN;
                for (uint32_t sl = 0; sl < nslices; ++sl, ++it) {
                    const uint32_t st = it % STAGES;
                    if (!mbar_wait(smem_addr(&full[st]), (it / STAGES) & 1u)) {
                        *failed = 1;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t a_base = smem_addr(a_slot(st)), b_base = smem_addr(b_slice(st, sl));
#pragma unroll
                    for (uint32_t j = 0; j < BK / 16; ++j) {
                        const uint64_t ad = smem_desc(a_base + 256u * j);
                        const uint64_t bd = smem_desc(b_base + 256u * j);
                        const uint32_t acc = (sl > 0 || j > 0) ? 1u : 0u;
                        asm volatile(
                            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(acc_addr),
                            "l"(ad), "l"(bd), "r"(IDESC), "r"(acc));
                    }
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                     smem_addr(&empty[st]))
                                 : "memory");
                }
                if (*failed) break;
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 smem_addr(&acc_full[b]))
                             : "memory");
            }
        }
        __syncwarp();
    } else {
        // epilogue: warp w reads accumulator lanes 32 (w % 4) .. + 31 (the lanes its position in
        // the warpgroup may address), columns 64 half .. + 63
        const uint32_t quarter = warp & 3u;
        const uint32_t half = (warp - (uint32_t)(PIPE_PRODUCERS + 1)) / 4u;
        drain_accumulators(g, tmem, acc_full, acc_empty, failed, ntiles, tiles_n, nslices, quarter, half, lane);
    }
    __syncthreads();
    if (*failed && threadIdx.x == 0 && err) atomicOr(err, DEVERR_MMA_TIMEOUT);
    if (warp == PIPE_PRODUCERS) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(PIPE_TMEM_COLS));
    }
}

// ---- TMA variant: plain row-major A and B^T, B resident ----------------------------------------
//
// For A without a row gather or a second source, and B^T of one column of tiles (n <= 128,
// k <= 64 RB_MAX_SLICES): one thread of warp 0 copies the operands with cp.async.bulk.tensor
// (TMA) in the 128-byte-swizzled K-major layout — B^T once per CTA (barrier `b_full`), then the
// A slices of the CTA's tiles into a 6-slot ring, each copy completing its slot's `full` barrier
// by its byte count (mbarrier expect_tx); warp 1 issues the MMAs with 128-byte-swizzle
// descriptors (a K step of 16 is a 32-byte advance inside the swizzle atom); warps 2..9 drain
// the accumulators as in gemm_pipe_kernel. The tensor maps cover this GPU's own global memory;
// no multicast.
constexpr int TMA_STAGES = 6;
constexpr int TMA_THREADS = 32 * (2 + PIPE_EPILOGUE);

// Shared-memory descriptor of a K-major operand tile in the 128-byte swizzle layout: rows of
// 128 bytes, 8-row groups 1,024 bytes apart (SBO), the leading-byte offset unused, version 1.
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(1024u >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

// One 64 x 128 box (64 K elements, 128 rows) of a 2-D BF16 tensor map into shared memory; the
// copy completes `bar` by its bytes. x (the K coordinate) is a multiple of 64 elements (128 B).
__device__ __forceinline__ void tma_load_box(const CUtensorMap* map, void* dst, uint32_t x, uint32_t y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_addr(bar))
        : "memory");
}

template <bool LN>
__global__ void __launch_bounds__(TMA_THREADS, 1) gemm_tma_kernel(const GemmArgs g,
                                                                  const __grid_constant__ CUtensorMap map_a,
                                                                  const __grid_constant__ CUtensorMap map_b,
                                                                  uint32_t* err) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    __shared__ uint64_t full[TMA_STAGES], empty[TMA_STAGES], acc_full[2], acc_empty[2], b_full;
    // LN: the warp pairs' exchanged row sums, squared deviations and wait outcomes
    __shared__ float s_lnx[LN ? 4 : 1][2][32], s_lnv[LN ? 4 : 1][2][32];
    __shared__ int s_lnok[LN ? 4 : 1][2];
    __shared__ uint32_t tmem_slot;
    __shared__ int s_failed;
    volatile int* failed = &s_failed;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t tiles_m = (g.m + BM - 1) / BM, tiles_n = 1u;
    const uint32_t ntiles = tiles_m;
    const uint32_t nslices = (g.k + BK - 1) / BK;
    // [B^T slices 0 .. nslices)[A ring], every slot 16 KB and 1,024-byte aligned
    unsigned char* const ring = smem_raw + nslices * TILE_BYTES;

    if (threadIdx.x == 0) {
        for (int q = 0; q < TMA_STAGES; ++q) {
            mbar_init(&full[q], 1);
            mbar_init(&empty[q], 1);
        }
        for (int q = 0; q < 2; ++q) {
            mbar_init(&acc_full[q], 1);
            mbar_init(&acc_empty[q], PIPE_EPILOGUE);
        }
        mbar_init(&b_full, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_failed = 0;
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(&tmem_slot)),
                     "r"(PIPE_TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            // B^T once, then the A slices of every tile through the ring
            mbar_expect_tx(&b_full, nslices * TILE_BYTES);
            for (uint32_t sl = 0; sl < nslices; ++sl) tma_load_box(&map_b, smem_raw + sl * TILE_BYTES, sl * BK, 0u, &b_full);
            uint32_t it = 0;
            for (uint32_t tile = blockIdx.x; tile < ntiles && !*failed; tile += gridDim.x) {
                const uint32_t m0 = tile * BM;
                for (uint32_t sl = 0; sl < nslices; ++sl, ++it) {
                    const uint32_t st = it % TMA_STAGES;
                    if (it >= (uint32_t)TMA_STAGES &&
                        !mbar_wait(smem_addr(&empty[st]), ((it / TMA_STAGES) - 1u) & 1u)) {
                        *failed = 1;
                        break;
                    }
                    mbar_expect_tx(&full[st], TILE_BYTES);
                    tma_load_box(&map_a, ring + st * TILE_BYTES, sl * BK, m0, &full[st]);
                }
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        // MMA issue (one thread)
        if (lane == 0) {
            uint32_t it = 0, t = 0;
            if (!mbar_wait(smem_addr(&b_full), 0u)) *failed = 1;
            for (uint32_t tile = blockIdx.x; tile < ntiles && !*failed; tile += gridDim.x, ++t) {
                const uint32_t b = t & 1u;
                if (t >= 2 && !mbar_wait(smem_addr(&acc_empty[b]), ((t >> 1) - 1u) & 1u)) {
                    *failed = 1;
                    break;
                }
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t acc_addr = tmem + b * (uint32_t)BN;
                for (uint32_t sl = 0; sl < nslices; ++sl, ++it) {
                    const uint32_t st = it % TMA_STAGES;
                    if (!mbar_wait(smem_addr(&full[st]), (it / TMA_STAGES) & 1u)) {
                        *failed = 1;
                        break;
                    }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t a_base = smem_addr(ring + st * TILE_BYTES);
                    const uint32_t b_base = smem_addr(smem_raw + sl * TILE_BYTES);
#pragma unroll
                    for (uint32_t j = 0; j < BK / 16; ++j) {
                        const uint64_t ad = sw128_desc(a_base + 32u * j);
                        const uint64_t bd = sw128_desc(b_base + 32u * j);
                        const uint32_t acc = (sl > 0 || j > 0) ? 1u : 0u;
                        asm volatile(
                            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(acc_addr),
                            "l"(ad), "l"(bd), "r"(IDESC), "r"(acc));
                    }
                    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                     smem_addr(&empty[st]))
                                 : "memory");
                }
                if (*failed) break;
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                                 smem_addr(&acc_full[b]))
                             : "memory");
            }
        }
        __syncwarp();
    } else {
        // warps 2..9: quarter w % 4, columns 64 ((w - 2) / 4) ..
        if constexpr (LN)
            drain_accumulators_ln(g, tmem, acc_full, acc_empty, failed, ntiles, nslices, warp & 3u, (warp - 2u) / 4u,
                                  lane, s_lnx, s_lnv, s_lnok);
        else
            drain_accumulators(g, tmem, acc_full, acc_empty, failed, ntiles, tiles_n, nslices, warp & 3u,
                               (warp - 2u) / 4u, lane);
    }
    __syncthreads();
    if (*failed && threadIdx.x == 0 && err) atomicOr(err, DEVERR_MMA_TIMEOUT);
    if (warp == 1) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(PIPE_TMEM_COLS));
    }
}

}  // namespace

// 64 KB of operand buffers: at most three CTAs per SM, 3 x 128 of the SM's 512 columns of
// tensor memory, so tcgen05.alloc never has to wait for another CTA.
size_t gemm_smem_bytes() { return 65u * 1024u; }

wc_status check_gemm(const GemmArgs& g) {
    if (g.m == 0 || g.n == 0) return WC_OK;
    if (!g.a || !g.b || (!g.c_f32 && !g.c_bf16)) return fail(WC_ERR_INVALID_ARG, "gemm: null operand");
    if (!g.a_transposed && (g.lda % 8 || (g.a2 && (g.lda2 % 8 || g.k_split % 8))))
        return fail(WC_ERR_INVALID_ARG, "gemm: row-major A needs 16-byte aligned rows (lda %% 8 == 0)");
    if (g.a_transposed && (g.lda % 8 || g.m % 8)) return fail(WC_ERR_INVALID_ARG, "gemm: transposed A needs m, lda %% 8 == 0");
    if (!g.b_rowmajor && g.ldb % 8) return fail(WC_ERR_INVALID_ARG, "gemm: B^T rows need ldb %% 8 == 0");
    if (g.b_rowmajor && (g.ldb % 8 || g.n % 8)) return fail(WC_ERR_INVALID_ARG, "gemm: row-major B needs n, ldb %% 8 == 0");
    // Both operands staged along k (transposed A, row-major B) read single k rows: any k works.
    if (g.k % 8 && !(g.a_transposed && g.b_rowmajor))
        return fail(WC_ERR_INVALID_ARG, "gemm: k must be a multiple of 8 (pad with zeros)");
    if ((g.add1 && !g.add1_idx) || (g.add2 && !g.add2_idx)) return fail(WC_ERR_INVALID_ARG, "gemm: gather without index");
    if (g.k_chunk == 0 || g.k_chunk % BK) return fail(WC_ERR_INVALID_ARG, "gemm: k_chunk must be a multiple of 64");
    if (g.ln_gamma && (g.n != 128u || !g.ln_beta || !g.c_bf16 || g.c_f32 || g.relu || g.add1 || g.add2 ||
                       g.accumulate || g.ldc != 128u || g.a_rows || g.a2 || g.a_transposed || g.b_rowmajor ||
                       g.k_chunk < g.k))
        return fail(WC_ERR_INVALID_ARG,
                    "gemm: the LayerNorm epilogue needs n = ldc = 128, beta, a BF16 output only and plain operands");
    return WC_OK;
}

// Dynamic shared memory of gemm_pipe_kernel<RB> for k (RB: the resident B slices and the ring).
size_t pipe_smem_bytes(bool rb, uint32_t k) {
    const uint32_t nslices = (k + BK - 1) / BK;
    return rb ? (size_t)(nslices + PipeShape<true>::STAGES) * TILE_BYTES
              : (size_t)PipeShape<false>::STAGES * 2u * TILE_BYTES;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (null when unavailable: the
// cp.async kernel then serves every shape).
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
    static const EncodeTiledFn fn = []() -> EncodeTiledFn {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            return nullptr;
        return reinterpret_cast<EncodeTiledFn>(p);
    }();
    return fn;
}

// A 2-D BF16 row-major tensor [outer x inner] with rows `stride_bytes` apart, read in boxes of
// 64 x 128 elements with the 128-byte swizzle, out-of-range elements as zeros.
bool encode_operand(CUtensorMap* map, const void* base, uint64_t inner, uint64_t outer, uint64_t stride_bytes) {
    const EncodeTiledFn fn = encode_tiled();
    if (!fn || reinterpret_cast<uintptr_t>(base) % 16u || stride_bytes % 16u || inner == 0 || outer == 0) return false;
    const cuuint64_t dims[2] = {inner, outer};
    const cuuint64_t strides[1] = {stride_bytes};
    const cuuint32_t box[2] = {(cuuint32_t)BK, (cuuint32_t)BM};
    const cuuint32_t elem[2] = {1, 1};
    return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, elem,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool gemm_ln_available() { return encode_tiled() != nullptr; }

wc_status launch_gemm(const GemmArgs& g, uint32_t* err, cudaStream_t s) {
    const wc_status st = check_gemm(g);
    if (st != WC_OK || g.m == 0 || g.n == 0) return st;
    if (!g.a_transposed && !g.b_rowmajor && g.k_chunk >= g.k) {
        // row-major operands, no split of K: the persistent pipelined kernel, one CTA per SM;
        // B resident in shared memory when it is one column of tiles of at most RB_MAX_SLICES
        static int sms = 0;
        if (!sms) {
            int dev = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
            if (sms <= 0) sms = 1;
            cudaFuncSetAttribute(gemm_pipe_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)pipe_smem_bytes(false, 0));
            cudaFuncSetAttribute(gemm_pipe_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)pipe_smem_bytes(true, RB_MAX_SLICES * BK));
        }
        const uint32_t tiles = ((g.m + BM - 1) / BM) * ((g.n + BN - 1) / BN);
        const uint32_t grid = tiles < (uint32_t)sms ? tiles : (uint32_t)sms;
        const bool rb = g.n <= (uint32_t)BN && (g.k + BK - 1) / BK <= RB_MAX_SLICES;
        if (rb && !g.a_rows && !g.a2) {
            // plain A: the TMA kernel, when both operands have tensor maps
            CUtensorMap ma, mb;
            if (encode_operand(&ma, g.a, g.k, g.m, 2ull * g.lda) && encode_operand(&mb, g.b, g.k, g.n, 2ull * g.ldb)) {
                static bool tma_attr = false;
                if (!tma_attr) {
                    cudaFuncSetAttribute(gemm_tma_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)pipe_smem_bytes(true, RB_MAX_SLICES * BK));
                    cudaFuncSetAttribute(gemm_tma_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)pipe_smem_bytes(true, RB_MAX_SLICES * BK));
                    tma_attr = true;
                }
                if (g.ln_gamma)
                    gemm_tma_kernel<true><<<grid, TMA_THREADS, pipe_smem_bytes(true, g.k), s>>>(g, ma, mb, err);
                else
                    gemm_tma_kernel<false><<<grid, TMA_THREADS, pipe_smem_bytes(true, g.k), s>>>(g, ma, mb, err);
                const cudaError_t e = cudaGetLastError();
                if (e != cudaSuccess) return fail(WC_ERR_CUDA, "gemm launch: %s", cudaGetErrorString(e));
                return WC_OK;
            }
        }
        if (g.ln_gamma) return fail(WC_ERR_STATE, "gemm: the LayerNorm epilogue needs the TMA kernel (plain A, k <= 384)");
        if (rb)
            gemm_pipe_kernel<true><<<grid, PIPE_THREADS, pipe_smem_bytes(true, g.k), s>>>(g, err);
        else
            gemm_pipe_kernel<false><<<grid, PIPE_THREADS, pipe_smem_bytes(false, g.k), s>>>(g, err);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return fail(WC_ERR_CUDA, "gemm launch: %s", cudaGetErrorString(e));
        return WC_OK;
    }
    static bool attr_done = false;
    if (!attr_done) {
        cudaFuncSetAttribute(gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gemm_smem_bytes());
        attr_done = true;
    }
    const dim3 grid((g.m + BM - 1) / BM, (g.n + BN - 1) / BN, (g.k + g.k_chunk - 1) / g.k_chunk);
    gemm_kernel<<<grid, THREADS, gemm_smem_bytes(), s>>>(g, err);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(WC_ERR_CUDA, "gemm launch: %s", cudaGetErrorString(e));
    return WC_OK;
}

}  // namespace nn
}  // namespace wc

extern "C" WC_API wc_status wc_nn_gemm(const wc_gemm_desc* d, uint32_t* d_err, void* stream) {
    wc::clear_error();
    if (!d) return wc::fail(WC_ERR_INVALID_ARG, "wc_nn_gemm: null descriptor");
    wc::nn::GemmArgs g{};
    g.m = d->m;
    g.n = d->n;
    g.k = d->k;
    g.k_chunk = d->k_chunk;
    g.a = static_cast<const __nv_bfloat16*>(d->a);
    g.a2 = static_cast<const __nv_bfloat16*>(d->a2);
    g.a_rows = d->a_rows;
    g.lda = d->lda;
    g.lda2 = d->lda2;
    g.k_split = d->k_split;
    g.a_transposed = d->a_transposed;
    g.b = static_cast<const __nv_bfloat16*>(d->b);
    g.ldb = d->ldb;
    g.b_rowmajor = d->b_rowmajor;
    g.bias = d->bias;
    g.add1 = static_cast<const __nv_bfloat16*>(d->add1);
    g.add1_idx = d->add1_idx;
    g.add2 = static_cast<const __nv_bfloat16*>(d->add2);
    g.add2_idx = d->add2_idx;
    g.ld_add = d->ld_add;
    g.relu = d->relu;
    g.c_f32 = d->c_f32;
    g.accumulate = d->accumulate;
    g.c_bf16 = static_cast<__nv_bfloat16*>(d->c_bf16);
    g.ldc = d->ldc;
    g.split_stride = d->split_stride;
    g.ln_gamma = d->ln_gamma;
    g.ln_beta = d->ln_beta;
    g.ln_resid = static_cast<const __nv_bfloat16*>(d->ln_resid);
    return wc::nn::launch_gemm(g, d_err, static_cast<cudaStream_t>(stream));
}
