// wc_surrogate.cu — the learned message-passing surrogate (no counterpart in the reference).
//
// Network (latent width 128, L message-passing steps, all GEMMs on the tensor cores):
//   node encoder  h0 = LN(W2 relu(W1 x_i + b1) + b2)          x_i: 5 velocities, 6 wall
//                                                              distances / h, k / rho0 (32)
//   edge encoder  e0 = LN(W2 relu(W1 f_ij + b1) + b2)         f_ij: (x_i - x_j)/h, |.|/h (16)
//   step l        e' = e + LN(W2 relu(W1 [e | h_i | h_j] + b1) + b2)
//                 h' = h + LN(W2 relu(W1 [h | sum_j e'_ij] + b1) + b2)
//   decoder       a_i = accel_scale (W2 relu(W1 h_i + b1) + b2)   (3 of 16 outputs used)
// The first edge layer is evaluated as W1e e + (W1i h)[receiver] + (W1s h)[sender]: the same
// linear map, with the two node terms computed once per node and gathered in the GEMM's
// epilogue. Edges are the radius-h pairs of the solver's cell tables, sorted by receiver, so the
// aggregation is a segment sum and the sender-side gradient a segment sum over reverse edges.
//
// Training: FP32 master weights, Adam, BF16 copies of every weight in both orientations
// (forward W^T, input-gradient W); gradients are FP32 and accumulate over the samples of a
// batch. The rollout runs plain SPH every K steps as the judge: it advances the state with both
// SPH and the surrogate, compares the two next states' SPH densities per particle, and keeps the
// surrogate's state only when the mean |rho_sur / rho_sph - 1| is within the tolerance.
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
using namespace wc::nn;

namespace {

constexpr uint32_t W = 128;  // latent width
constexpr uint32_t NODE_IN = 32, EDGE_IN = 16, OUT = 16;
constexpr size_t NONE = ~size_t(0);

struct Lin {
    size_t w = 0, b = NONE;  // FP32 offsets (w: [kin x nout] row-major)
    uint32_t kin = 0, nout = 0;
    size_t wt = 0, wk = 0;   // BF16 offsets: W^T [nout x kin], W [kin x nout]
};
struct LNp {
    size_t g = 0;  // gamma at g, beta at g + 128
};
struct MPLayer {
    Lin e1e, e1i, e1s, e2, n1, n2;
    LNp lne, lnn;
};

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

inline uint64_t splitmix64(uint64_t& st) {
    uint64_t z = (st += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Activations of one graph. `saved` keeps every layer's (training); otherwise two buffers
// alternate (inference on graphs too large to keep all layers).
struct Work {
    uint32_t cap_n = 0, cap_e = 0, layers = 0;
    bool saved = false;
    // graph
    uint32_t *rowptr = nullptr, *col = nullptr, *recv = nullptr, *rev = nullptr, *count = nullptr;
    uint32_t *scan_scratch = nullptr, *scan_words = nullptr;
    unsigned long long* scan_desc = nullptr;
    // inputs (sorted order)
    float4 *hist_s = nullptr, *target_s = nullptr, *stale_s = nullptr;
    __nv_bfloat16 *xn = nullptr, *xe = nullptr;
    // node side
    __nv_bfloat16 *h = nullptr, *zn0 = nullptr, *P = nullptr, *Q = nullptr, *agg = nullptr, *zn = nullptr, *zd = nullptr;
    float *yn0 = nullptr, *yn = nullptr, *out = nullptr, *stn0 = nullptr, *stn = nullptr;
    // edge side
    __nv_bfloat16 *e = nullptr, *ze0 = nullptr, *ze = nullptr;
    float *ye0 = nullptr, *ye = nullptr, *ste0 = nullptr, *ste = nullptr;
    // gradients
    float *dh = nullptr, *dagg = nullptr, *dtmp_n = nullptr, *dP = nullptr, *dQ = nullptr, *dout = nullptr;
    float *de = nullptr, *dtmp_e = nullptr;
    __nv_bfloat16 *gb_n = nullptr, *gb_n2 = nullptr, *gb_e = nullptr, *dout_b = nullptr, *dPb = nullptr, *dQb = nullptr;
    float *part = nullptr;  // split-K partials / column-sum partials
    size_t part_cap = 0;
    float* loss_part = nullptr;
};

void free_work(Work& w) {
    void* ptrs[] = {w.stale_s, w.rowptr, w.col,  w.recv, w.rev,  w.count, w.scan_scratch, w.scan_words, w.scan_desc, w.hist_s,
                    w.target_s, w.xn, w.xe,   w.h,    w.zn0,   w.P,            w.Q,          w.agg,       w.zn,
                    w.zd,     w.yn0,  w.yn,   w.out,  w.stn0,  w.stn,          w.e,          w.ze0,       w.ze,
                    w.ye0,    w.ye,   w.ste0, w.ste,  w.dh,    w.dagg,         w.dtmp_n,     w.dP,        w.dQ,
                    w.dout,   w.de,   w.dtmp_e, w.gb_n, w.gb_n2, w.gb_e,       w.dout_b,     w.dPb,       w.dQb,
                    w.part,   w.loss_part};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    w = Work{};
}

}  // namespace

struct wc_surrogate {
    wc_surrogate_config cfg{};
    uint32_t L = 8;
    Lin ne1, ne2, ee1, ee2, d1, d2;
    LNp lnn0, lne0;
    std::vector<MPLayer> layers;
    size_t nparams = 0, nbf16 = 0;
    float *w = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
    __nv_bfloat16* wb = nullptr;
    int adam_step = 0;
    bool cast_dirty = true;
    Work work;
    cudaStream_t stream = nullptr;
    uint32_t* d_err = nullptr;
    uint32_t* h_err = nullptr;
    // current sample
    wc_fluid* fluid = nullptr;
    uint32_t n = 0, e = 0;
    bool has_target = false;
    bool has_stale = false;  // the loaded sample is residual: its outputs are added to work.stale_s
    float dt = 1e-3f;  // time step of the loaded sample (velocity differences / dt are features)
    float4* hist_in = nullptr;  // [5 n] in state order (sample / rollout history)
    float4* target_in = nullptr;
    float4* stale_in = nullptr;  // [n] last SPH acceleration of a sample, state order
    uint32_t cap_in = 0;
    // rollout scratch
    float4 *save_pos = nullptr, *save_vel = nullptr, *alt_pos = nullptr, *alt_vel = nullptr;
    float4 *stale = nullptr, *stale_tmp = nullptr;  // last SPH acceleration (stale-acceleration mode)
    float *rho_a = nullptr, *rho_b = nullptr;
    double* err_part = nullptr;
    uint32_t cap_roll = 0;
};

namespace {

size_t alloc_f(wc_surrogate* s, size_t count) {
    const size_t off = s->nparams;
    s->nparams += (count + 3) & ~size_t(3);
    return off;
}
size_t alloc_b(wc_surrogate* s, size_t count) {
    const size_t off = s->nbf16;
    s->nbf16 += (count + 7) & ~size_t(7);
    return off;
}
Lin make_lin(wc_surrogate* s, uint32_t kin, uint32_t nout, bool bias) {
    Lin l;
    l.kin = kin;
    l.nout = nout;
    l.w = alloc_f(s, (size_t)kin * nout);
    if (bias) l.b = alloc_f(s, nout);
    l.wt = alloc_b(s, (size_t)kin * nout);
    l.wk = alloc_b(s, (size_t)kin * nout);
    return l;
}
LNp make_ln(wc_surrogate* s) { return LNp{alloc_f(s, 2 * W)}; }

template <class F>
void for_each_lin(wc_surrogate* s, F f) {
    for (Lin* l : {&s->ne1, &s->ne2, &s->ee1, &s->ee2, &s->d1, &s->d2}) f(*l);
    for (MPLayer& L : s->layers)
        for (Lin* l : {&L.e1e, &L.e1i, &L.e1s, &L.e2, &L.n1, &L.n2}) f(*l);
}
template <class F>
void for_each_ln(wc_surrogate* s, F f) {
    f(s->lnn0);
    f(s->lne0);
    for (MPLayer& L : s->layers) {
        f(L.lne);
        f(L.lnn);
    }
}

void init_params(wc_surrogate* s, std::vector<float>& host) {
    host.assign(s->nparams, 0.f);
    uint64_t st = s->cfg.seed;
    for_each_lin(s, [&](Lin& l) {
        // uniform(-a, a) with a = sqrt(6 / (fan_in + fan_out)) (Glorot)
        const float a = std::sqrt(6.0f / (float)(l.kin + l.nout));
        for (size_t i = 0; i < (size_t)l.kin * l.nout; ++i)
            host[l.w + i] = a * (2.0f * (float)((splitmix64(st) >> 40) * (1.0 / 16777216.0)) - 1.0f);
    });
    // the decoder's output layer starts small; only 3 of its 16 outputs are used
    for (size_t k = 0; k < s->d2.kin; ++k)
        for (size_t n = 0; n < s->d2.nout; ++n) host[s->d2.w + k * s->d2.nout + n] *= n < 3 ? 0.1f : 0.0f;
    for_each_ln(s, [&](LNp& ln) {
        for (uint32_t i = 0; i < W; ++i) host[ln.g + i] = 1.0f;
    });
}

void cast_all(wc_surrogate* s) {
    for_each_lin(s, [&](Lin& l) { cast_weight(s->w + l.w, l.kin, l.nout, l.kin, l.nout, s->wb + l.wt, s->wb + l.wk, s->stream); });
    s->cast_dirty = false;
}

// ---- GEMM helpers ------------------------------------------------------------------------------

wc_status fwd(wc_surrogate* s, const Lin& l, uint32_t rows, const __nv_bfloat16* a, const __nv_bfloat16* a2,
              bool relu, float* c_f32, __nv_bfloat16* c_bf16, const __nv_bfloat16* add1 = nullptr,
              const uint32_t* i1 = nullptr, const __nv_bfloat16* add2 = nullptr, const uint32_t* i2 = nullptr,
              bool with_bias = true) {
    GemmArgs g{};
    g.m = rows;
    g.n = l.nout;
    g.k = l.kin;
    g.k_chunk = ((l.kin + 63) / 64) * 64;
    g.a = a;
    g.lda = a2 ? l.kin / 2 : l.kin;
    if (a2) {
        g.a2 = a2;
        g.lda2 = l.kin / 2;
        g.k_split = l.kin / 2;
    }
    g.b = s->wb + l.wt;
    g.ldb = l.kin;
    g.bias = (with_bias && l.b != NONE) ? s->w + l.b : nullptr;
    g.add1 = add1;
    g.add1_idx = i1;
    g.add2 = add2;
    g.add2_idx = i2;
    g.ld_add = l.nout;
    g.relu = relu;
    g.c_f32 = c_f32;
    g.c_bf16 = c_bf16;
    g.ldc = l.nout;
    return launch_gemm(g, s->d_err, s->stream);
}

// out = LN(a . W^T + b) * gamma + beta (+ resid) in one GEMM with the LayerNorm in its epilogue
// (the forward pass of a rollout, which keeps no activations for a backward pass).
wc_status fwd_ln(wc_surrogate* s, const Lin& l, uint32_t rows, const __nv_bfloat16* a, const float* gamma,
                 const __nv_bfloat16* resid, __nv_bfloat16* out) {
    GemmArgs g{};
    g.m = rows;
    g.n = l.nout;
    g.k = l.kin;
    g.k_chunk = ((l.kin + 63) / 64) * 64;
    g.a = a;
    g.lda = l.kin;
    g.b = s->wb + l.wt;
    g.ldb = l.kin;
    g.bias = l.b != NONE ? s->w + l.b : nullptr;
    g.c_bf16 = out;
    g.ldc = l.nout;
    g.ln_gamma = gamma;
    g.ln_beta = gamma + W;
    g.ln_resid = resid;
    return launch_gemm(g, s->d_err, s->stream);
}

// dX (rows x kcount) (+)= dY . W[k0 : k0 + kcount]^T
wc_status dgrad(wc_surrogate* s, const Lin& l, uint32_t rows, const __nv_bfloat16* dy, uint32_t k0, uint32_t kcount,
                float* dx, bool accumulate) {
    GemmArgs g{};
    g.m = rows;
    g.n = kcount;
    g.k = l.nout;
    g.k_chunk = ((l.nout + 63) / 64) * 64;
    g.a = dy;
    g.lda = l.nout;
    g.b = s->wb + l.wk + (size_t)k0 * l.nout;
    g.ldb = l.nout;
    g.c_f32 = dx;
    g.accumulate = accumulate;
    g.ldc = kcount;
    return launch_gemm(g, s->d_err, s->stream);
}

wc_status ensure_part(wc_surrogate* s, size_t count) {
    Work& w = s->work;
    if (count <= w.part_cap) return WC_OK;
    dfree(w.part);
    WC_TRY(dalloc(&w.part, count));
    w.part_cap = count;
    return WC_OK;
}

// grad W[k0 : k0 + kcount] += X^T dY over `rows` rows (split over the rows, partials reduced in
// a fixed order).
wc_status wgrad(wc_surrogate* s, const Lin& l, uint32_t rows, const __nv_bfloat16* x, uint32_t kcount, uint32_t k0,
                const __nv_bfloat16* dy) {
    if (!rows) return WC_OK;
    uint32_t chunk = ((rows / 256 + 63) / 64) * 64;
    if (chunk < 1024) chunk = 1024;
    const uint32_t splits = (rows + chunk - 1) / chunk;
    const size_t tile = (size_t)kcount * l.nout;
    WC_TRY(ensure_part(s, splits * tile));
    GemmArgs g{};
    g.m = kcount;
    g.n = l.nout;
    g.k = rows;
    g.k_chunk = chunk;
    g.a = x;
    g.lda = kcount;
    g.a_transposed = 1;
    g.b = dy;
    g.ldb = l.nout;
    g.b_rowmajor = 1;
    g.c_f32 = s->work.part;
    g.ldc = l.nout;
    g.split_stride = tile;
    WC_TRY(launch_gemm(g, s->d_err, s->stream));
    colsum_partials(splits, (uint32_t)tile, s->work.part, s->g + l.w + (size_t)k0 * l.nout, 1, s->stream);
    return WC_OK;
}

wc_status bgrad(wc_surrogate* s, const Lin& l, uint32_t rows, const float* dy) {
    if (l.b == NONE || !rows) return WC_OK;
    WC_TRY(ensure_part(s, (size_t)colsum_blocks(rows) * l.nout));
    colsum(rows, l.nout, l.nout, dy, s->work.part, s->g + l.b, 1, s->stream);
    return WC_OK;
}

wc_status ln_back(wc_surrogate* s, const LNp& ln, uint32_t rows, const float* dout, const float* y, const float* st,
                  __nv_bfloat16* dy, float* dy_f32) {
    const uint32_t blocks = layernorm_backward_blocks(rows);
    if (!blocks) return WC_OK;
    WC_TRY(ensure_part(s, (size_t)blocks * 256));
    layernorm_backward(rows, dout, y, st, st + rows, s->w + ln.g, dy, dy_f32, s->work.part, s->stream);
    colsum_partials(blocks, 256, s->work.part, s->g + ln.g, 1, s->stream);
    return WC_OK;
}

// ---- workspace -------------------------------------------------------------------------------

wc_status ensure_work(wc_surrogate* s, uint32_t n, uint32_t e, bool saved) {
    Work& w = s->work;
    if (n <= w.cap_n && e <= w.cap_e && (saved == w.saved || !saved) && w.layers == s->L) return WC_OK;
    const size_t part_cap = w.part_cap;
    free_work(w);
    const uint32_t cn = std::max(n, 1u), ce = std::max(e, 1u);
    const size_t Ls = saved ? s->L : 2, Ln = saved ? s->L + 1 : 2;
    w.cap_n = cn;
    w.cap_e = ce;
    w.saved = saved;
    w.layers = s->L;
    const size_t tiles = ((size_t)cn + 1 + SCAN_TILE - 1) / SCAN_TILE;
    WC_TRY(dalloc(&w.rowptr, (size_t)cn + 1));
    WC_TRY(dalloc(&w.count, (size_t)cn + 1));
    WC_TRY(dalloc(&w.scan_scratch, (size_t)cn + 1));
    WC_TRY(dalloc(&w.scan_words, 4));
    WC_TRY(dalloc(&w.scan_desc, tiles));
    WC_TRY(dalloc(&w.col, ce));
    WC_TRY(dalloc(&w.recv, ce));
    WC_TRY(dalloc(&w.rev, ce));
    WC_TRY(dalloc(&w.hist_s, 5 * (size_t)cn));
    WC_TRY(dalloc(&w.target_s, cn));
    WC_TRY(dalloc(&w.stale_s, cn));
    WC_TRY(dalloc(&w.xn, (size_t)cn * NODE_IN));
    WC_TRY(dalloc(&w.xe, (size_t)ce * EDGE_IN));
    WC_TRY(dalloc(&w.h, Ln * cn * W));
    WC_TRY(dalloc(&w.zn0, (size_t)cn * W));
    WC_TRY(dalloc(&w.yn0, (size_t)cn * W));
    WC_TRY(dalloc(&w.stn0, 2 * (size_t)cn));
    WC_TRY(dalloc(&w.P, (size_t)cn * W));
    WC_TRY(dalloc(&w.Q, (size_t)cn * W));
    WC_TRY(dalloc(&w.agg, Ls * cn * W));
    WC_TRY(dalloc(&w.zn, Ls * cn * W));
    WC_TRY(dalloc(&w.yn, Ls * cn * W));
    WC_TRY(dalloc(&w.stn, Ls * 2 * cn));
    WC_TRY(dalloc(&w.zd, (size_t)cn * W));
    WC_TRY(dalloc(&w.out, (size_t)cn * OUT));
    WC_TRY(dalloc(&w.e, Ln * ce * W));
    WC_TRY(dalloc(&w.ze0, (size_t)ce * W));
    WC_TRY(dalloc(&w.ye0, (size_t)ce * W));
    WC_TRY(dalloc(&w.ste0, 2 * (size_t)ce));
    WC_TRY(dalloc(&w.ze, Ls * ce * W));
    WC_TRY(dalloc(&w.ye, Ls * ce * W));
    WC_TRY(dalloc(&w.ste, Ls * 2 * ce));
    WC_TRY(dalloc(&w.loss_part, mse_blocks(cn) + 1));
    if (saved) {
        WC_TRY(dalloc(&w.dh, (size_t)cn * W));
        WC_TRY(dalloc(&w.dagg, (size_t)cn * W));
        WC_TRY(dalloc(&w.dtmp_n, (size_t)cn * W));
        WC_TRY(dalloc(&w.dP, (size_t)cn * W));
        WC_TRY(dalloc(&w.dQ, (size_t)cn * W));
        WC_TRY(dalloc(&w.dout, (size_t)cn * OUT));
        WC_TRY(dalloc(&w.de, (size_t)ce * W));
        WC_TRY(dalloc(&w.dtmp_e, (size_t)ce * W));
        WC_TRY(dalloc(&w.gb_n, (size_t)cn * W));
        WC_TRY(dalloc(&w.gb_n2, (size_t)cn * W));
        WC_TRY(dalloc(&w.gb_e, (size_t)ce * W));
        WC_TRY(dalloc(&w.dout_b, (size_t)cn * OUT));
        WC_TRY(dalloc(&w.dPb, (size_t)cn * W));
        WC_TRY(dalloc(&w.dQb, (size_t)cn * W));
    }
    // split-K partials of the weight gradients (<= 257 splits of a 128 x 128 tile), column-sum
    // and LayerNorm-backward partials
    size_t need = std::max<size_t>(part_cap, 257u * (size_t)W * W);
    need = std::max<size_t>(need, (size_t)layernorm_backward_blocks(ce) * 256);
    need = std::max<size_t>(need, (size_t)colsum_blocks(ce) * W);
    WC_TRY(ensure_part(s, need));
    return WC_OK;
}

__nv_bfloat16* hbuf(Work& w, uint32_t l) { return w.h + (size_t)(w.saved ? l : (l & 1u)) * w.cap_n * W; }
__nv_bfloat16* ebuf(Work& w, uint32_t l) { return w.e + (size_t)(w.saved ? l : (l & 1u)) * w.cap_e * W; }
template <class T>
T* lbuf(Work& w, T* base, uint32_t l, size_t per) { return base + (size_t)(w.saved ? l : 0u) * per; }

// ---- graph from a sorted fluid ------------------------------------------------------------------

// The radius-h graph of the fluid's sorted buffer (its tables must match it): per-particle
// neighbour counts, an exclusive scan (the cell scan kernel reused over particles), the
// neighbour lists (ascending slots), receivers and reverse edges.
wc_status build_graph(wc_surrogate* s, const FluidInternals& fi, uint32_t* e_out, bool saved) {
    const DevBuffers& d = *fi.d;
    const SceneConsts& sc = *fi.sc;
    const uint32_t n = d.n;
    // The edge count is only known after the count pass: size the node side first.
    WC_TRY(ensure_work(s, n, std::max(s->work.cap_e, 1u), saved));
    Work& w = s->work;
    graph_count(d.pos_b, n, d.start, sc.bin, sc.R, sc.cull, w.count, s->d_err, s->stream);
    DevBuffers sd{};
    sd.n = n;
    sd.num_cells = n;
    sd.num_tiles = (n + SCAN_TILE - 1) / SCAN_TILE;
    sd.counts = w.count;
    sd.start = w.rowptr;
    sd.cell_list = w.scan_scratch;
    sd.num_nonempty = w.scan_words + 1;
    sd.scan_desc = w.scan_desc;
    sd.scan_tile_counter = w.scan_words;
    sd.err = s->d_err;
    WC_CUDA_TRY(cudaMemsetAsync(w.scan_desc, 0, sizeof(unsigned long long) * std::max(sd.num_tiles, 1u), s->stream));
    WC_CUDA_TRY(cudaMemsetAsync(w.scan_words, 0, sizeof(uint32_t), s->stream));
    if (n) launch_scan_cells(sd, s->stream);
    uint32_t e = 0;
    if (n) WC_CUDA_TRY(cudaMemcpyAsync(&e, w.rowptr + n, sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream));
    WC_CUDA_TRY(cudaStreamSynchronize(s->stream));
    if (e > w.cap_e) {
        // grow the edge side (keeps nothing of this graph but the scan, which is recomputed)
        WC_TRY(ensure_work(s, n, e + e / 8, saved));
        return build_graph(s, fi, e_out, saved);
    }
    graph_fill(d.pos_b, n, d.start, sc.bin, sc.R, sc.cull, w.rowptr, w.col, s->stream);
    graph_rev(n, w.rowptr, w.col, w.recv, w.rev, s->stream);
    *e_out = e;
    return WC_OK;
}

// Features of the sorted sample: hist_s/target_s are gathered by the sort's permutation. `stale`
// (the last SPH acceleration, `age` steps old; null for none) is in the state order, or already
// in the sorted order when stale_sorted. A sample with a stale acceleration is residual: the
// network's output is the change since then (the loss target is target - stale), and the
// acceleration it stands for is stale + output (added in FP32, so the large part of the
// acceleration never passes through the BF16 network).
wc_status prepare_sample(wc_surrogate* s, wc_fluid* f, bool saved, const float4* stale = nullptr,
                         bool stale_sorted = false, uint32_t age = 0) {
    FluidInternals fi = fluid_internals(f);
    const DevBuffers& d = *fi.d;
    uint32_t e = 0;
    WC_TRY(build_graph(s, fi, &e, saved));
    Work& w = s->work;
    const uint32_t n = d.n;
    for (int k = 0; k < 5; ++k) gather4(n, d.perm, s->hist_in + (size_t)k * n, w.hist_s + (size_t)k * n, s->stream);
    if (s->has_target) gather4(n, d.perm, s->target_in, w.target_s, s->stream);
    const float k_feature = fi.params->stiffness / fi.params->rest_density * 200.0f;
    const float inv_dv = 1.0f / (s->dt * s->cfg.accel_scale);
    const float4* stale_sorted_buf = nullptr;
    if (stale && age > 0) {
        if (stale_sorted) {
            stale_sorted_buf = stale;
        } else {
            gather4(n, d.perm, stale, w.stale_s, s->stream);
            stale_sorted_buf = w.stale_s;
        }
        if (s->has_target) sub_xyz(n, w.target_s, stale_sorted_buf, s->stream);
    }
    s->has_stale = stale_sorted_buf != nullptr && !stale_sorted;
    node_features(n, d.pos_b, w.hist_s, 1.0f / s->cfg.velocity_scale, inv_dv, 1.0f / fi.sc->h, fi.sc->size, k_feature,
                  stale_sorted_buf, 1.0f / s->cfg.accel_scale, (float)age * 0.125f, w.xn, s->stream);
    edge_features(e, d.pos_b, w.recv, w.col, 1.0f / fi.sc->h, w.xe, s->stream);
    s->n = n;
    s->e = e;
    return WC_OK;
}

// ---- forward / backward ---------------------------------------------------------------------

// keep: the activations and LayerNorm statistics the backward pass reads (training); without
// it every second MLP layer and its LayerNorm run as one GEMM with the LayerNorm in the epilogue.
wc_status forward(wc_surrogate* s, bool keep) {
    if (s->cast_dirty) cast_all(s);
    Work& w = s->work;
    const uint32_t n = s->n, e = s->e;
    const bool fuse = !keep && gemm_ln_available();
    float* st = w.stn0;
    WC_TRY(fwd(s, s->ne1, n, w.xn, nullptr, true, nullptr, w.zn0));
    if (fuse) {
        WC_TRY(fwd_ln(s, s->ne2, n, w.zn0, s->w + s->lnn0.g, nullptr, hbuf(w, 0)));
    } else {
        WC_TRY(fwd(s, s->ne2, n, w.zn0, nullptr, false, w.yn0, nullptr));
        layernorm(n, w.yn0, s->w + s->lnn0.g, s->w + s->lnn0.g + W, nullptr, hbuf(w, 0), st, st + n, s->stream);
    }
    WC_TRY(fwd(s, s->ee1, e, w.xe, nullptr, true, nullptr, w.ze0));
    if (fuse) {
        WC_TRY(fwd_ln(s, s->ee2, e, w.ze0, s->w + s->lne0.g, nullptr, ebuf(w, 0)));
    } else {
        WC_TRY(fwd(s, s->ee2, e, w.ze0, nullptr, false, w.ye0, nullptr));
        layernorm(e, w.ye0, s->w + s->lne0.g, s->w + s->lne0.g + W, nullptr, ebuf(w, 0), w.ste0, w.ste0 + e,
                  s->stream);
    }
    const size_t pn = (size_t)w.cap_n * W, pe = (size_t)w.cap_e * W;
    for (uint32_t l = 0; l < s->L; ++l) {
        const MPLayer& L = s->layers[l];
        __nv_bfloat16 *h = hbuf(w, l), *h1 = hbuf(w, l + 1), *el = ebuf(w, l), *e1 = ebuf(w, l + 1);
        __nv_bfloat16* ze = lbuf(w, w.ze, l, pe);
        float* ye = lbuf(w, w.ye, l, pe);
        float* ste = lbuf(w, w.ste, l, 2 * (size_t)w.cap_e);
        __nv_bfloat16* agg = lbuf(w, w.agg, l, pn);
        __nv_bfloat16* zn = lbuf(w, w.zn, l, pn);
        float* yn = lbuf(w, w.yn, l, pn);
        float* stn = lbuf(w, w.stn, l, 2 * (size_t)w.cap_n);
        WC_TRY(fwd(s, L.e1i, n, h, nullptr, false, nullptr, w.P));
        WC_TRY(fwd(s, L.e1s, n, h, nullptr, false, nullptr, w.Q));
        WC_TRY(fwd(s, L.e1e, e, el, nullptr, true, nullptr, ze, w.P, w.recv, w.Q, w.col));
        if (fuse) {
            WC_TRY(fwd_ln(s, L.e2, e, ze, s->w + L.lne.g, el, e1));
        } else {
            WC_TRY(fwd(s, L.e2, e, ze, nullptr, false, ye, nullptr));
            layernorm(e, ye, s->w + L.lne.g, s->w + L.lne.g + W, el, e1, ste, ste + e, s->stream);
        }
        segment_sum_bf16(n, w.rowptr, nullptr, e1, nullptr, agg, s->stream);
        WC_TRY(fwd(s, L.n1, n, h, agg, true, nullptr, zn));
        if (fuse) {
            WC_TRY(fwd_ln(s, L.n2, n, zn, s->w + L.lnn.g, h, h1));
        } else {
            WC_TRY(fwd(s, L.n2, n, zn, nullptr, false, yn, nullptr));
            layernorm(n, yn, s->w + L.lnn.g, s->w + L.lnn.g + W, h, h1, stn, stn + n, s->stream);
        }
    }
    WC_TRY(fwd(s, s->d1, n, hbuf(w, s->L), nullptr, true, nullptr, w.zd));
    WC_TRY(fwd(s, s->d2, n, w.zd, nullptr, false, w.out, nullptr));
    return WC_OK;
}

wc_status backward(wc_surrogate* s) {
    Work& w = s->work;
    const uint32_t n = s->n, e = s->e;
    const size_t pn = (size_t)w.cap_n * W, pe = (size_t)w.cap_e * W;
    // decoder
    WC_TRY(wgrad(s, s->d2, n, w.zd, W, 0, w.dout_b));
    WC_TRY(bgrad(s, s->d2, n, w.dout));
    WC_TRY(dgrad(s, s->d2, n, w.dout_b, 0, W, w.dtmp_n, false));
    relu_mask((size_t)n * W, w.dtmp_n, w.zd, w.gb_n, s->stream);
    WC_TRY(wgrad(s, s->d1, n, hbuf(w, s->L), W, 0, w.gb_n));
    WC_TRY(bgrad(s, s->d1, n, w.dtmp_n));
    WC_TRY(dgrad(s, s->d1, n, w.gb_n, 0, W, w.dh, false));
    WC_CUDA_TRY(cudaMemsetAsync(w.de, 0, sizeof(float) * (size_t)e * W, s->stream));
    for (int li = (int)s->L - 1; li >= 0; --li) {
        const uint32_t l = (uint32_t)li;
        const MPLayer& L = s->layers[l];
        __nv_bfloat16 *h = hbuf(w, l), *el = ebuf(w, l);
        __nv_bfloat16* ze = lbuf(w, w.ze, l, pe);
        float* ye = lbuf(w, w.ye, l, pe);
        float* ste = lbuf(w, w.ste, l, 2 * (size_t)w.cap_e);
        __nv_bfloat16* agg = lbuf(w, w.agg, l, pn);
        __nv_bfloat16* zn = lbuf(w, w.zn, l, pn);
        float* yn = lbuf(w, w.yn, l, pn);
        float* stn = lbuf(w, w.stn, l, 2 * (size_t)w.cap_n);
        // node block: h' = h + LN(yn); dh holds d h' and keeps flowing to h (residual)
        WC_TRY(ln_back(s, L.lnn, n, w.dh, yn, stn, w.gb_n, w.dtmp_n));
        WC_TRY(wgrad(s, L.n2, n, zn, W, 0, w.gb_n));
        WC_TRY(bgrad(s, L.n2, n, w.dtmp_n));
        WC_TRY(dgrad(s, L.n2, n, w.gb_n, 0, W, w.dtmp_n, false));
        relu_mask((size_t)n * W, w.dtmp_n, zn, w.gb_n2, s->stream);  // gb_n2 = d zn
        WC_TRY(wgrad(s, L.n1, n, h, W, 0, w.gb_n2));
        WC_TRY(wgrad(s, L.n1, n, agg, W, W, w.gb_n2));
        WC_TRY(bgrad(s, L.n1, n, w.dtmp_n));
        WC_TRY(dgrad(s, L.n1, n, w.gb_n2, 0, W, w.dh, true));
        WC_TRY(dgrad(s, L.n1, n, w.gb_n2, W, W, w.dagg, false));
        // edge block: e' = e + LN(ye); de holds d e' from the next layer, plus the aggregation
        gather_add(e, w.recv, w.dagg, w.de, s->stream);
        WC_TRY(ln_back(s, L.lne, e, w.de, ye, ste, w.gb_e, w.dtmp_e));
        WC_TRY(wgrad(s, L.e2, e, ze, W, 0, w.gb_e));
        WC_TRY(bgrad(s, L.e2, e, w.dtmp_e));
        WC_TRY(dgrad(s, L.e2, e, w.gb_e, 0, W, w.dtmp_e, false));
        relu_mask((size_t)e * W, w.dtmp_e, ze, w.gb_e, s->stream);  // gb_e = d ze
        WC_TRY(wgrad(s, L.e1e, e, el, W, 0, w.gb_e));
        WC_TRY(bgrad(s, L.e1e, e, w.dtmp_e));
        WC_TRY(dgrad(s, L.e1e, e, w.gb_e, 0, W, w.de, true));
        segment_sum_f32(n, w.rowptr, nullptr, w.dtmp_e, w.dP, w.dPb, s->stream);
        segment_sum_f32(n, w.rowptr, w.rev, w.dtmp_e, w.dQ, w.dQb, s->stream);
        WC_TRY(wgrad(s, L.e1i, n, h, W, 0, w.dPb));
        WC_TRY(wgrad(s, L.e1s, n, h, W, 0, w.dQb));
        WC_TRY(dgrad(s, L.e1i, n, w.dPb, 0, W, w.dh, true));
        WC_TRY(dgrad(s, L.e1s, n, w.dQb, 0, W, w.dh, true));
    }
    // encoders
    WC_TRY(ln_back(s, s->lnn0, n, w.dh, w.yn0, w.stn0, w.gb_n, w.dtmp_n));
    WC_TRY(wgrad(s, s->ne2, n, w.zn0, W, 0, w.gb_n));
    WC_TRY(bgrad(s, s->ne2, n, w.dtmp_n));
    WC_TRY(dgrad(s, s->ne2, n, w.gb_n, 0, W, w.dtmp_n, false));
    relu_mask((size_t)n * W, w.dtmp_n, w.zn0, w.gb_n, s->stream);
    WC_TRY(wgrad(s, s->ne1, n, w.xn, NODE_IN, 0, w.gb_n));
    WC_TRY(bgrad(s, s->ne1, n, w.dtmp_n));
    WC_TRY(ln_back(s, s->lne0, e, w.de, w.ye0, w.ste0, w.gb_e, w.dtmp_e));
    WC_TRY(wgrad(s, s->ee2, e, w.ze0, W, 0, w.gb_e));
    WC_TRY(bgrad(s, s->ee2, e, w.dtmp_e));
    WC_TRY(dgrad(s, s->ee2, e, w.gb_e, 0, W, w.dtmp_e, false));
    relu_mask((size_t)e * W, w.dtmp_e, w.ze0, w.gb_e, s->stream);
    WC_TRY(wgrad(s, s->ee1, e, w.xe, EDGE_IN, 0, w.gb_e));
    WC_TRY(bgrad(s, s->ee1, e, w.dtmp_e));
    return WC_OK;
}

wc_status read_err(wc_surrogate* s) {
    WC_CUDA_TRY(cudaStreamSynchronize(s->stream));
    WC_CUDA_TRY(cudaMemcpy(s->h_err, s->d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    if (*s->h_err) {
        cudaMemset(s->d_err, 0, sizeof(uint32_t));
        if (*s->h_err & DEVERR_CELL_OVERFLOW)
            return fail(WC_ERR_NUMERIC, "a cell row held more than %u particles (a collapsed or non-finite state)",
                        3u * MAX_CELL_PARTICLES);
        return fail(WC_ERR_TIMEOUT, "a tensor-core GEMM or scan wait exceeded its limit (flags %u)", *s->h_err);
    }
    return WC_OK;
}

wc_status ensure_inputs(wc_surrogate* s, uint32_t n) {
    if (n <= s->cap_in) return WC_OK;
    dfree(s->hist_in);
    dfree(s->target_in);
    dfree(s->stale_in);
    WC_TRY(dalloc(&s->hist_in, 5 * (size_t)n));
    WC_TRY(dalloc(&s->target_in, n));
    WC_TRY(dalloc(&s->stale_in, n));
    s->cap_in = n;
    return WC_OK;
}

// FP64 totals of one fluid's state: mass, momentum, kinetic and potential energy.
__global__ void fluid_diag_kernel(uint32_t n, const float4* __restrict__ pos, const float4* __restrict__ vel, double m,
                                  float gx, float gy, float gz, double* __restrict__ part) {
    __shared__ double sacc[5][256];
    double a[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 v = vel[i], p = pos[i];
        a[0] += m * v.x;
        a[1] += m * v.y;
        a[2] += m * v.z;
        a[3] += 0.5 * m * ((double)v.x * v.x + (double)v.y * v.y + (double)v.z * v.z);
        a[4] -= m * ((double)gx * p.x + (double)gy * p.y + (double)gz * p.z);
    }
    for (int q = 0; q < 5; ++q) sacc[q][threadIdx.x] = a[q];
    __syncthreads();
    for (int h = 128; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h)
            for (int q = 0; q < 5; ++q) sacc[q][threadIdx.x] += sacc[q][threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int q = 0; q < 5; ++q) part[(size_t)blockIdx.x * 5 + q] = sacc[q][0];
}

}  // namespace

wc_status wc::fluid_diagnostics(wc_fluid* f, double out[6]) {
    FluidInternals fi = fluid_internals(f);
    const uint32_t blocks = 256;
    double* part = nullptr;
    WC_TRY(dalloc(&part, blocks * 5));
    fluid_diag_kernel<<<blocks, 256, 0, fi.stream>>>(fi.d->n, fi.d->pos_a, fi.d->vel_a, (double)fi.params->particle_mass,
                                                     fi.in->g[0], fi.in->g[1], fi.in->g[2], part);
    std::vector<double> h(blocks * 5);
    cudaMemcpyAsync(h.data(), part, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, fi.stream);
    cudaStreamSynchronize(fi.stream);
    cudaFree(part);
    out[0] = (double)fi.params->particle_mass * fi.d->n;
    for (int q = 0; q < 5; ++q) {
        double a = 0.0;
        for (uint32_t b = 0; b < blocks; ++b) a += h[(size_t)b * 5 + q];
        out[1 + q] = a;
    }
    return WC_OK;
}

namespace {

// history (state order) <- [v_new, gathered history shifted by one] (sorted order of this step)
__global__ void shift_history_kernel(uint32_t n, const float4* __restrict__ vel, const float4* __restrict__ hs,
                                     float4* __restrict__ hist) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    hist[i] = vel[i];
#pragma unroll
    for (int k = 1; k < 5; ++k) hist[(size_t)k * n + i] = hs[(size_t)(k - 1) * n + i];
}


// One judged rollout (surrogate or stale-acceleration mode) on the fluid's stream.
struct RolloutRun {
    wc_surrogate* s;
    wc_fluid* f;
    FluidInternals fi;
    float dt;
    uint32_t K;
    float tolerance;
    int mode;
    wc_rollout_stats* out;
    const float* host_hist;  // initial velocity history, or null
    LaunchDims dims{};
    uint32_t age = 0;  // steps since the SPH acceleration in s->stale was computed
    double err_sum = 0.0, err_max = 0.0;

    wc_status copy(float4* dst, const float4* src) {
        WC_CUDA_TRY(cudaMemcpyAsync(dst, src, sizeof(float4) * fi.d->n, cudaMemcpyDeviceToDevice, fi.stream));
        return WC_OK;
    }

    // The candidate next state of the current state (network or stale acceleration), written to
    // (dst_pos, dst_vel) in the order of the current state's sort.
    wc_status candidate(float4* dst_pos, float4* dst_vel) {
        DevBuffers& D = *fi.d;
        fluid_enqueue_sort(f);
        const float* acc;
        uint32_t ld;
        float scale;
        if (mode == WC_ROLLOUT_SURROGATE || mode == WC_ROLLOUT_HYBRID) {
            if (mode == WC_ROLLOUT_HYBRID) {
                // the last SPH acceleration, in this step's sorted order, as network input; the
                // step's acceleration is that plus the network's residual (work.stale_s is free
                // in a rollout: the stale input is already sorted)
                gather4(D.n, D.perm, s->stale, s->stale_tmp, fi.stream);
                WC_TRY(prepare_sample(s, f, false, s->stale_tmp, true, age));
                WC_TRY(forward(s, false));
                add_scaled(D.n, s->work.out, OUT, s->cfg.accel_scale, s->stale_tmp, s->work.stale_s, fi.stream);
                acc = reinterpret_cast<const float*>(s->work.stale_s);
                ld = 4;
                scale = 1.0f;
            } else {
                WC_TRY(prepare_sample(s, f, false));
                WC_TRY(forward(s, false));
                acc = s->work.out;
                ld = OUT;
                scale = s->cfg.accel_scale;
            }
        } else {
            gather4(D.n, D.perm, s->stale, s->stale_tmp, fi.stream);
            acc = reinterpret_cast<const float*>(s->stale_tmp);
            ld = 4;
            scale = 1.0f;
        }
        DevBuffers tgt = D;
        tgt.pos_a = dst_pos;
        tgt.vel_a = dst_vel;
        // A candidate written beside the state buffer leaves its ids alone: they must keep
        // matching the state's particles, which the judge's SPH step sorts next.
        if (dst_pos != D.pos_a) tgt.ids_a = nullptr;
        integrate(D.n, *fi.sc, dt, acc, ld, scale, tgt, fi.stream);
        return WC_OK;
    }

    // SPH density of the state buffer, per state slot.
    void densities(float* rho) {
        DevBuffers& D = *fi.d;
        fluid_enqueue_sort(f);
        launch_density(D, *fi.sc, dims, fi.stream);
        scatter_density(D.n, D.perm, D.pos_b, rho, fi.stream);
    }

    void shift_history() {
        // the candidate step gathered the history in this step's order
        const uint32_t n = fi.d->n;
        shift_history_kernel<<<(n + 255) / 256, 256, 0, fi.stream>>>(n, fi.d->vel_a, s->work.hist_s, s->hist_in);
    }

    wc_status judge_step() {
        DevBuffers& D = *fi.d;
        const uint32_t n = D.n;
        WC_TRY(candidate(s->alt_pos, s->alt_vel));  // the state buffer is left as it was
        WC_TRY(fluid_graph_step(f, dt));             // SPH next state, in the same sorted order
        if (mode != WC_ROLLOUT_SURROGATE) WC_TRY(copy(s->stale, D.accel));
        WC_TRY(copy(s->save_pos, D.pos_a));
        WC_TRY(copy(s->save_vel, D.vel_a));
        densities(s->rho_a);
        WC_TRY(copy(D.pos_a, s->alt_pos));
        WC_TRY(copy(D.vel_a, s->alt_vel));
        densities(s->rho_b);
        rel_err(n, s->rho_b, s->rho_a, s->err_part, fi.stream);
        std::vector<double> parts(rel_err_blocks(n));
        if (n)
            WC_CUDA_TRY(cudaMemcpyAsync(parts.data(), s->err_part, sizeof(double) * parts.size(), cudaMemcpyDeviceToHost,
                                        fi.stream));
        WC_CUDA_TRY(cudaStreamSynchronize(fi.stream));
        double acc = 0.0;
        for (double p : parts) acc += p;
        const double err = n ? acc / n : 0.0;
        err_sum += err;
        err_max = std::max(err_max, err);
        ++out->judged;
        ++out->sph_steps;
        if (!(err <= tolerance)) {
            ++out->reverted;
            WC_TRY(copy(D.pos_a, s->save_pos));
            WC_TRY(copy(D.vel_a, s->save_vel));
        } else {
            ++out->surrogate_steps;
        }
        if (mode != WC_ROLLOUT_STALE) shift_history();
        age = 1;  // the judge's SPH acceleration is the one the next step sees
        return WC_OK;
    }

    wc_status go(uint32_t nsteps) {
        DevBuffers& D = *fi.d;
        const uint32_t n = D.n;
        int device = 0;
        WC_CUDA_TRY(cudaGetDevice(&device));
        dims = compute_launch_dims(device);
        if (host_hist) {
            WC_CUDA_TRY(cudaMemcpyAsync(s->hist_in, host_hist, sizeof(float4) * 5 * (size_t)n, cudaMemcpyHostToDevice,
                                        fi.stream));
        } else {
            // history starts as five copies of the current velocity
            for (int k = 0; k < 5; ++k) WC_TRY(copy(s->hist_in + (size_t)k * n, D.vel_a));
        }
        s->has_target = false;
        cudaEvent_t e0, e1;
        WC_CUDA_TRY(cudaEventCreate(&e0));
        WC_CUDA_TRY(cudaEventCreate(&e1));
        const auto t0 = std::chrono::steady_clock::now();
        cudaEventRecord(e0, fi.stream);
        wc_status rc = WC_OK;
        for (uint32_t step = 0; step < nsteps && rc == WC_OK; ++step) {
            if (mode != WC_ROLLOUT_SURROGATE && step == 0) {
                // no SPH acceleration yet: one plain step records it
                rc = fluid_graph_step(f, dt);
                if (rc == WC_OK) rc = copy(s->stale, D.accel);
                if (rc == WC_OK && mode == WC_ROLLOUT_HYBRID) {
                    // the history gains the step's velocity in its order (the sort's permutation)
                    rc = ensure_work(s, D.n, std::max(s->work.cap_e, 1u), false);
                }
                if (rc == WC_OK && mode == WC_ROLLOUT_HYBRID) {
                    for (int k = 0; k < 4; ++k)
                        gather4(D.n, D.perm, s->hist_in + (size_t)k * D.n, s->work.hist_s + (size_t)k * D.n, fi.stream);
                    shift_history();
                }
                age = 1;
                ++out->sph_steps;
            } else if (step % K == 0) {
                rc = judge_step();
            } else {
                rc = candidate(D.pos_a, D.vel_a);
                if (mode != WC_ROLLOUT_SURROGATE) std::swap(s->stale, s->stale_tmp);
                if (rc == WC_OK && mode != WC_ROLLOUT_STALE) shift_history();
                ++age;
                ++out->surrogate_steps;
            }
            fluid_count_step(f);
            ++out->steps;
        }
        cudaEventRecord(e1, fi.stream);
        const cudaError_t ce = cudaStreamSynchronize(fi.stream);
        const auto t1 = std::chrono::steady_clock::now();
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (rc != WC_OK) return rc;
        if (ce != cudaSuccess) return fail(WC_ERR_CUDA, "rollout: %s", cudaGetErrorString(ce));
        out->ms_device = ms;
        out->ms_wall = std::chrono::duration<double, std::milli>(t1 - t0).count();
        out->particle_steps_per_s = ms > 0 ? (double)n * out->steps / (ms * 1e-3) : 0.0;
        out->mean_density_error = out->judged ? err_sum / out->judged : 0.0;
        out->max_density_error = err_max;
        return WC_OK;
    }
};

}  // namespace

extern "C" {

WC_API void wc_surrogate_config_default(wc_surrogate_config* c) {
    if (!c) return;
    std::memset(c, 0, sizeof *c);
    c->layers = 8;
    c->seed = 1;
    c->velocity_scale = 1.0f;
    c->accel_scale = 10.0f;
}

WC_API wc_status wc_surrogate_create(const wc_surrogate_config* c, wc_surrogate** out) {
    clear_error();
    if (!c || !out) return fail(WC_ERR_INVALID_ARG, "null argument");
    if (c->layers == 0 || c->layers > 32) return fail(WC_ERR_INVALID_ARG, "layers must be in 1..32");
    if (!(c->velocity_scale > 0.f) || !(c->accel_scale > 0.f)) return fail(WC_ERR_INVALID_ARG, "scales must be > 0");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return fail(WC_ERR_CUDA, "no CUDA device");
    wc_surrogate* s = new (std::nothrow) wc_surrogate();
    if (!s) return fail(WC_ERR_OOM, "host allocation failed");
    s->cfg = *c;
    s->L = c->layers;
    s->ne1 = make_lin(s, NODE_IN, W, true);
    s->ne2 = make_lin(s, W, W, true);
    s->lnn0 = make_ln(s);
    s->ee1 = make_lin(s, EDGE_IN, W, true);
    s->ee2 = make_lin(s, W, W, true);
    s->lne0 = make_ln(s);
    s->layers.resize(s->L);
    for (MPLayer& L : s->layers) {
        L.e1e = make_lin(s, W, W, true);
        L.e1i = make_lin(s, W, W, false);
        L.e1s = make_lin(s, W, W, false);
        L.e2 = make_lin(s, W, W, true);
        L.lne = make_ln(s);
        L.n1 = make_lin(s, 2 * W, W, true);
        L.n2 = make_lin(s, W, W, true);
        L.lnn = make_ln(s);
    }
    s->d1 = make_lin(s, W, W, true);
    s->d2 = make_lin(s, W, OUT, true);
    wc_status st = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) == cudaSuccess
                       ? WC_OK
                       : fail(WC_ERR_CUDA, "stream creation failed");
    if (st == WC_OK) st = dalloc(&s->w, s->nparams);
    if (st == WC_OK) st = dalloc(&s->g, s->nparams);
    if (st == WC_OK) st = dalloc(&s->m, s->nparams);
    if (st == WC_OK) st = dalloc(&s->v, s->nparams);
    if (st == WC_OK) st = dalloc(&s->wb, s->nbf16);
    if (st == WC_OK) st = dalloc(&s->d_err, 1);
    if (st == WC_OK && cudaMallocHost(reinterpret_cast<void**>(&s->h_err), sizeof(uint32_t)) != cudaSuccess)
        st = fail(WC_ERR_OOM, "pinned allocation failed");
    if (st == WC_OK) {
        std::vector<float> host;
        init_params(s, host);
        cudaMemcpy(s->w, host.data(), sizeof(float) * s->nparams, cudaMemcpyHostToDevice);
        cudaMemset(s->g, 0, sizeof(float) * s->nparams);
        cudaMemset(s->m, 0, sizeof(float) * s->nparams);
        cudaMemset(s->v, 0, sizeof(float) * s->nparams);
        cudaMemset(s->d_err, 0, sizeof(uint32_t));
        const cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) st = fail(WC_ERR_CUDA, "surrogate init: %s", cudaGetErrorString(e));
    }
    if (st != WC_OK) {
        wc_surrogate_destroy(s);
        return st;
    }
    *out = s;
    return WC_OK;
}

WC_API void wc_surrogate_destroy(wc_surrogate* s) {
    if (!s) return;
    if (s->stream) cudaStreamSynchronize(s->stream);
    free_work(s->work);
    void* ptrs[] = {s->w, s->g, s->m, s->v, s->wb, s->d_err, s->hist_in, s->target_in, s->stale_in, s->save_pos, s->save_vel,
                    s->alt_pos, s->alt_vel, s->stale, s->stale_tmp, s->rho_a, s->rho_b, s->err_part};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (s->h_err) cudaFreeHost(s->h_err);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

WC_API uint64_t wc_surrogate_num_params(const wc_surrogate* s) { return s ? s->nparams : 0; }

WC_API wc_status wc_surrogate_get_params(wc_surrogate* s, float* host, uint64_t n) {
    clear_error();
    if (!s || !host || n != s->nparams) return fail(WC_ERR_INVALID_ARG, "parameter buffer must hold %llu floats",
                                                    (unsigned long long)(s ? s->nparams : 0));
    WC_CUDA_TRY(cudaStreamSynchronize(s->stream));
    WC_CUDA_TRY(cudaMemcpy(host, s->w, sizeof(float) * n, cudaMemcpyDeviceToHost));
    return WC_OK;
}

WC_API wc_status wc_surrogate_set_params(wc_surrogate* s, const float* host, uint64_t n) {
    clear_error();
    if (!s || !host || n != s->nparams) return fail(WC_ERR_INVALID_ARG, "parameter buffer must hold %llu floats",
                                                    (unsigned long long)(s ? s->nparams : 0));
    WC_CUDA_TRY(cudaStreamSynchronize(s->stream));
    WC_CUDA_TRY(cudaMemcpy(s->w, host, sizeof(float) * n, cudaMemcpyHostToDevice));
    s->cast_dirty = true;
    return WC_OK;
}

WC_API wc_status wc_surrogate_get_grads(wc_surrogate* s, float* host, uint64_t n) {
    clear_error();
    if (!s || !host || n != s->nparams) return fail(WC_ERR_INVALID_ARG, "gradient buffer size");
    WC_TRY(read_err(s));
    WC_CUDA_TRY(cudaMemcpy(host, s->g, sizeof(float) * n, cudaMemcpyDeviceToHost));
    return WC_OK;
}

WC_API wc_status wc_surrogate_zero_grads(wc_surrogate* s) {
    clear_error();
    if (!s) return fail(WC_ERR_INVALID_ARG, "null surrogate");
    WC_CUDA_TRY(cudaMemsetAsync(s->g, 0, sizeof(float) * s->nparams, s->stream));
    return WC_OK;
}

WC_API wc_status wc_surrogate_sample(wc_surrogate* s, wc_fluid* f, float dt, const float* host_hist,
                                     const float* host_target, const float* host_stale, uint32_t stale_age) {
    clear_error();
    WC_NVTX("wc_surrogate_sample");
    if (!s || !f || !host_hist) return fail(WC_ERR_INVALID_ARG, "null argument");
    if (!(dt > 0.f)) return fail(WC_ERR_INVALID_ARG, "dt must be > 0");
    s->dt = dt;
    FluidInternals fi = fluid_internals(f);
    const uint32_t n = fi.d->n;
    WC_TRY(ensure_inputs(s, n));
    // The fluid's stream and the surrogate's must not overlap: order them through host syncs.
    WC_CUDA_TRY(cudaStreamSynchronize(fi.stream));
    WC_CUDA_TRY(cudaMemcpyAsync(s->hist_in, host_hist, sizeof(float4) * 5 * (size_t)n, cudaMemcpyHostToDevice, s->stream));
    s->has_target = host_target != nullptr;
    if (host_target)
        WC_CUDA_TRY(cudaMemcpyAsync(s->target_in, host_target, sizeof(float4) * n, cudaMemcpyHostToDevice, s->stream));
    const bool stale = host_stale != nullptr && stale_age > 0;
    if (stale)
        WC_CUDA_TRY(cudaMemcpyAsync(s->stale_in, host_stale, sizeof(float4) * n, cudaMemcpyHostToDevice, s->stream));
    WC_CUDA_TRY(cudaStreamSynchronize(s->stream));
    fluid_enqueue_sort(f);
    WC_CUDA_TRY(cudaStreamSynchronize(fi.stream));
    WC_TRY(prepare_sample(s, f, true, stale ? s->stale_in : nullptr, false, stale ? stale_age : 0u));
    s->fluid = f;
    return read_err(s);
}

WC_API wc_status wc_surrogate_forward_backward(wc_surrogate* s, int do_backward, double* loss) {
    clear_error();
    WC_NVTX("wc_surrogate_forward_backward");
    if (!s || !s->fluid) return fail(WC_ERR_STATE, "no sample loaded (wc_surrogate_sample)");
    if (do_backward && !s->has_target) return fail(WC_ERR_STATE, "backward needs a sample with targets");
    WC_TRY(forward(s, do_backward != 0));
    Work& w = s->work;
    if (s->has_target) {
        mse(s->n, OUT, w.out, w.target_s, 1.0f / s->cfg.accel_scale, do_backward ? w.dout : nullptr,
            do_backward ? w.dout_b : nullptr, w.loss_part, s->stream);
        if (do_backward) WC_TRY(backward(s));
        if (loss) {
            const uint32_t blocks = mse_blocks(s->n);
            std::vector<float> parts(blocks);
            WC_CUDA_TRY(cudaMemcpyAsync(parts.data(), w.loss_part, sizeof(float) * blocks, cudaMemcpyDeviceToHost,
                                        s->stream));
            WC_TRY(read_err(s));
            double acc = 0.0;
            for (float p : parts) acc += p;
            *loss = s->n ? acc / (3.0 * s->n) : 0.0;
        }
    }
    return read_err(s);
}

WC_API wc_status wc_surrogate_predictions(wc_surrogate* s, float* host_out, uint32_t n) {
    clear_error();
    if (!s || !s->fluid || !host_out || n != s->n) return fail(WC_ERR_INVALID_ARG, "prediction buffer must hold n x 4");
    // outputs are in sorted order: undo the sample's permutation on the host
    FluidInternals fi = fluid_internals(s->fluid);
    std::vector<float> out((size_t)n * OUT);
    std::vector<uint32_t> perm(n);
    std::vector<float4> base(s->has_stale ? n : 0);
    WC_CUDA_TRY(cudaMemcpyAsync(out.data(), s->work.out, sizeof(float) * out.size(), cudaMemcpyDeviceToHost, s->stream));
    WC_CUDA_TRY(cudaMemcpyAsync(perm.data(), fi.d->perm, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, s->stream));
    if (s->has_stale)
        WC_CUDA_TRY(cudaMemcpyAsync(base.data(), s->work.stale_s, sizeof(float4) * n, cudaMemcpyDeviceToHost, s->stream));
    WC_TRY(read_err(s));
    for (uint32_t k = 0; k < n; ++k) {
        const float b[3] = {s->has_stale ? base[k].x : 0.f, s->has_stale ? base[k].y : 0.f,
                            s->has_stale ? base[k].z : 0.f};
        for (int a = 0; a < 4; ++a)
            host_out[(size_t)perm[k] * 4 + a] = a < 3 ? std::fmaf(out[(size_t)k * OUT + a], s->cfg.accel_scale, b[a]) : 0.f;
    }
    return WC_OK;
}

WC_API wc_status wc_surrogate_adam(wc_surrogate* s, float lr, float grad_scale) {
    clear_error();
    WC_NVTX("wc_surrogate_adam");
    if (!s) return fail(WC_ERR_INVALID_ARG, "null surrogate");
    ++s->adam_step;
    adam(s->nparams, s->w, s->g, s->m, s->v, lr, 0.9f, 0.999f, 1e-8f, s->adam_step, grad_scale, s->stream);
    WC_CUDA_TRY(cudaMemsetAsync(s->g, 0, sizeof(float) * s->nparams, s->stream));
    s->cast_dirty = true;
    return read_err(s);
}

WC_API wc_status wc_surrogate_rollout(wc_surrogate* s, wc_fluid* f, float dt, uint32_t nsteps, uint32_t K,
                                      float tolerance, int mode, const float* hist, wc_rollout_stats* out) {
    clear_error();
    WC_NVTX("wc_surrogate_rollout");
    if (!out) return fail(WC_ERR_INVALID_ARG, "null argument");
    std::memset(out, 0, sizeof *out);
    if (!f || (mode != WC_ROLLOUT_SPH && !s)) return fail(WC_ERR_INVALID_ARG, "null argument");
    if (mode != WC_ROLLOUT_SPH && mode != WC_ROLLOUT_SURROGATE && mode != WC_ROLLOUT_STALE &&
        mode != WC_ROLLOUT_HYBRID)
        return fail(WC_ERR_INVALID_ARG, "unknown rollout mode %d", mode);
    if (K == 0) return fail(WC_ERR_INVALID_ARG, "K must be >= 1");
    if (mode == WC_ROLLOUT_SPH) {
        // plain SPH: the graph-launched solver, timed like the other modes
        FluidInternals fi = fluid_internals(f);
        WC_CUDA_TRY(cudaStreamSynchronize(fi.stream));
        WC_TRY(fluid_diagnostics(f, out->diag_start));
        cudaEvent_t e0, e1;
        WC_CUDA_TRY(cudaEventCreate(&e0));
        WC_CUDA_TRY(cudaEventCreate(&e1));
        const auto t0 = std::chrono::steady_clock::now();
        cudaEventRecord(e0, fi.stream);
        wc_status rc = WC_OK;
        for (uint32_t step = 0; step < nsteps && rc == WC_OK; ++step) {
            rc = fluid_graph_step(f, dt);
            fluid_count_step(f);
        }
        cudaEventRecord(e1, fi.stream);
        const cudaError_t ce = cudaStreamSynchronize(fi.stream);
        const auto t1 = std::chrono::steady_clock::now();
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (rc != WC_OK) return rc;
        if (ce != cudaSuccess) return fail(WC_ERR_CUDA, "rollout: %s", cudaGetErrorString(ce));
        out->steps = out->sph_steps = nsteps;
        out->ms_device = ms;
        out->ms_wall = std::chrono::duration<double, std::milli>(t1 - t0).count();
        out->particle_steps_per_s = ms > 0 ? (double)fi.d->n * nsteps / (ms * 1e-3) : 0.0;
        return fluid_diagnostics(f, out->diag_end);
    }
    FluidInternals fi = fluid_internals(f);
    const uint32_t n = fi.d->n;
    WC_TRY(ensure_inputs(s, n));
    if (n > s->cap_roll) {
        for (float4** p : {&s->save_pos, &s->save_vel, &s->alt_pos, &s->alt_vel, &s->stale, &s->stale_tmp})
            dfree(*p);
        dfree(s->rho_a);
        dfree(s->rho_b);
        dfree(s->err_part);
        s->cap_roll = 0;
        WC_TRY(dalloc(&s->save_pos, n));
        WC_TRY(dalloc(&s->save_vel, n));
        WC_TRY(dalloc(&s->alt_pos, n));
        WC_TRY(dalloc(&s->alt_vel, n));
        WC_TRY(dalloc(&s->stale, n));
        WC_TRY(dalloc(&s->stale_tmp, n));
        WC_TRY(dalloc(&s->rho_a, n));
        WC_TRY(dalloc(&s->rho_b, n));
        WC_TRY(dalloc(&s->err_part, rel_err_blocks(n) + 1));
        s->cap_roll = n;
    }
    const bool was_recording = fi.d->accel != nullptr;
    const bool needs_accel = mode == WC_ROLLOUT_STALE || mode == WC_ROLLOUT_HYBRID;
    if (needs_accel && !was_recording) WC_TRY(wc_fluid_set_recording(f, 1));
    WC_CUDA_TRY(cudaStreamSynchronize(fi.stream));
    WC_TRY(fluid_diagnostics(f, out->diag_start));
    cudaStream_t own = s->stream;
    s->stream = fi.stream;  // everything runs on the fluid's stream
    s->dt = dt;
    RolloutRun run{s, f, fi, dt, K, tolerance, mode, out, hist};
    const wc_status rc = run.go(nsteps);
    s->stream = own;
    s->fluid = nullptr;  // the loaded sample was replaced by the rollout's graphs
    if (needs_accel && !was_recording) wc_fluid_set_recording(f, 0);
    if (rc != WC_OK) return rc;
    WC_TRY(read_err(s));
    return fluid_diagnostics(f, out->diag_end);
}

}  // extern "C"
