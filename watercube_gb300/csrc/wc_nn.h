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
    __nv_bfloat16* c_bf16;
    uint32_t ldc;
    size_t split_stride;
};

size_t gemm_smem_bytes();
wc_status check_gemm(const GemmArgs& g);
wc_status launch_gemm(const GemmArgs& g, uint32_t* err, cudaStream_t s);

}  // namespace nn
}  // namespace wc
