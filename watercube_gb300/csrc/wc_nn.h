// wc_nn.h — kernels of the learned surrogate (message passing on the radius-h graph).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/watercube.h"

namespace wc {
namespace nn {

// C = A . B (+ bias) (+ add1[add1_idx[row]] + add2[add2_idx[row]]) (ReLU), see wc_nn_gemm.cu.
struct GemmArgs {
    uint32_t m, n, k;
    uint32_t k_chunk;  // K range per blockIdx.z (split-K); partial results land split_stride apart
    const __nv_bfloat16* a;
    const __nv_bfloat16* a2;  // second A source for columns >= k_split, or null
    const uint32_t* a_rows;   // A row gather, or null
    uint32_t lda, lda2, k_split;
    int a_transposed;         // A[i][kk] = a[kk * lda + i]
    const __nv_bfloat16* b;
    uint32_t ldb;
    int b_rowmajor;           // 0: b is B^T [n x k]; 1: b is B [k x n]
    const float* bias;
    const __nv_bfloat16* add1;
    const uint32_t* add1_idx;
    const __nv_bfloat16* add2;
    const uint32_t* add2_idx;
    uint32_t ld_add;
    int relu;
    float* c_f32;
    int accumulate;  // c_f32 += result instead of =
    __nv_bfloat16* c_bf16;
    uint32_t ldc;
    size_t split_stride;
    // LayerNorm epilogue (ln_gamma set): c_bf16 = LN(result) * ln_gamma + ln_beta (+ ln_resid rows)
    const float* ln_gamma;
    const float* ln_beta;
    const __nv_bfloat16* ln_resid;
};

size_t gemm_smem_bytes();
// Whether launch_gemm can run a LayerNorm-epilogue GEMM (the TMA kernel's tensor maps exist).
bool gemm_ln_available();
wc_status check_gemm(const GemmArgs& g);
wc_status launch_gemm(const GemmArgs& g, uint32_t* err, cudaStream_t s);

}  // namespace nn
}  // namespace wc

// ---- non-GEMM kernels (wc_nn_ops.cu) -----------------------------------------------------------
namespace wc {
struct SceneConsts;
struct DevBuffers;
namespace nn {

void graph_count(const float4* pos, uint32_t n, const uint32_t* start, float bin, int32_t R, float cull,
                 uint32_t* count, uint32_t* err, cudaStream_t s);
void graph_fill(const float4* pos, uint32_t n, const uint32_t* start, float bin, int32_t R, float cull,
                const uint32_t* rowptr, uint32_t* col, cudaStream_t s);
void graph_rev(uint32_t n, const uint32_t* rowptr, const uint32_t* col, uint32_t* recv, uint32_t* rev, cudaStream_t s);
void node_features(uint32_t n, const float4* pos, const float4* hist, float inv_v, float inv_dv, float inv_h,
                   float size, float k_feature, const float4* stale, float inv_a, float age_feature,
                   __nv_bfloat16* out, cudaStream_t s);
void edge_features(uint32_t e, const float4* pos, const uint32_t* recv, const uint32_t* col, float inv_h,
                   __nv_bfloat16* out, cudaStream_t s);
void layernorm(uint32_t rows, const float* y, const float* gamma, const float* beta, const __nv_bfloat16* resid,
               __nv_bfloat16* out, float* mean, float* rstd, cudaStream_t s);
uint32_t layernorm_backward_blocks(uint32_t rows);
void layernorm_backward(uint32_t rows, const float* dout, const float* y, const float* mean, const float* rstd,
                        const float* gamma, __nv_bfloat16* dy, float* dy_f32, float* part, cudaStream_t s);
void relu_mask(size_t count, float* g_inout, const __nv_bfloat16* z, __nv_bfloat16* out, cudaStream_t s);
void cast_bf16(size_t count, const float* x, __nv_bfloat16* out, cudaStream_t s);
void gather_add(uint32_t rows, const uint32_t* idx, const float* src, float* dst, cudaStream_t s);
void segment_sum_bf16(uint32_t nodes, const uint32_t* rowptr, const uint32_t* idx, const __nv_bfloat16* src,
                      float* out_f32, __nv_bfloat16* out_bf16, cudaStream_t s);
void segment_sum_f32(uint32_t nodes, const uint32_t* rowptr, const uint32_t* idx, const float* src, float* out_f32,
                     __nv_bfloat16* out_bf16, cudaStream_t s);
uint32_t colsum_blocks(uint32_t rows);
void colsum(uint32_t rows, uint32_t cols, uint32_t ld, const float* x, float* part, float* out, int accumulate,
            cudaStream_t s);
void colsum_partials(uint32_t blocks, uint32_t cols, const float* part, float* out, int accumulate, cudaStream_t s);
uint32_t mse_blocks(uint32_t n);
void mse(uint32_t n, uint32_t ldp, const float* pred, const float4* target, float inv_scale, float* dpred_f32,
         __nv_bfloat16* dpred, float* part, cudaStream_t s);
void adam(size_t count, float* w, const float* g, float* m, float* v, float lr, float b1, float b2, float eps,
          int step, float grad_scale, cudaStream_t s);
void cast_weight(const float* w, uint32_t k_in, uint32_t n_out, uint32_t k_pad, uint32_t n_pad, __nv_bfloat16* wt,
                 __nv_bfloat16* wk, cudaStream_t s);
void gather4(uint32_t n, const uint32_t* perm, const float4* src, float4* dst, cudaStream_t s);
void sub_xyz(uint32_t n, float4* dst, const float4* sub, cudaStream_t s);
void add_scaled(uint32_t n, const float* pred, uint32_t ldp, float scale, const float4* base, float4* dst,
                cudaStream_t s);
void scatter_density(uint32_t n, const uint32_t* ids, const float4* src, float* dst, cudaStream_t s);
uint32_t rel_err_blocks(uint32_t n);
void rel_err(uint32_t n, const float* a, const float* b, double* part, cudaStream_t s);
// A surrogate step's integrator: sorted buffer (B) + predicted acceleration -> state buffer (A).
void integrate(uint32_t n, const SceneConsts& sc, float dt, const float* pred, uint32_t ldp, float a_scale,
               const DevBuffers& d, cudaStream_t s);

}  // namespace nn
}  // namespace wc
