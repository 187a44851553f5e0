// gemm_tc.cuh -- BF16 conditioner path (tcgen05/TMEM GEMMs fed by TMA, gemm_tc.cu).
#pragma once
#include <cuda_bf16.h>
#include "flow.cuh"

namespace fmc {

namespace tc {
// epilogues of the tensor-core GEMM: 0 tanh(acc + bias) -> bf16;
// 1 acc + bias -> fp32; 2 acc * (1 - aux^2) -> bf16 (tanh adjoint, aux = the
// forward's tanh output); 3 acc -> fp32 (no bias).
enum Epi : int { TC_EPI_TANH_BF16 = 0, TC_EPI_BIAS_F32 = 1, TC_EPI_DTANH_BF16 = 2, TC_EPI_F32 = 3 };

struct EpiArgs {
  const float* bias;        // modes 0, 1
  const uint16_t* aux;      // mode 2: bf16 [M, ldaux]
  int64_t ldaux;
  float* kpart;             // mode 3: optional scratch for split-K partial products
  int64_t kpart_floats;     //   (the GEMM splits K when the tile grid leaves SMs idle)
  float* colpart;           // mode 2 with TMA stores: column sums of the bf16 output per
  int64_t ldpart;           //   32-row block, row (m / 32) of colpart [ceil(M / 128) * 4, ldpart]
  int rmap_grp, rmap_keep;  // fp32 modes: output row m goes to (m / grp) * keep + m % grp and is
                            //   dropped when m % grp >= keep (grp = 0: rows as they are)
  int kslices;              // mode 3 with kpart: K slices asked for (0 = enough to fill the SMs)
};
}  // namespace tc

__device__ __forceinline__ uint16_t f32_to_bf16_rn(float v) {
  return __bfloat16_as_ushort(__float2bfloat16_rn(v));
}

size_t train_ws_bytes(const FlowGeom& g, int64_t n, bool bf16);

// the conditioner's hidden layers only (conversion + tanh GEMMs); *h_last is
// the last tanh activation (bf16 [round_up(m, 128), round_up(H_last, 64)]);
// with cond == NULL, cond16 already holds the bf16 conditioning block
int conditioner_bf16_hidden(const FmcFlow* f, const FlowGeom& g, int l, int64_t m, const float* cond,
                            uint16_t* cond16, uint16_t* h16a, uint16_t* h16b, const uint16_t** h_last,
                            cudaStream_t st);

// epilogue warps per TMEM lane quarter in the fused spline kernel; each
// leaves one log-determinant partial per row and coordinate group
constexpr int kSplineEpiPerQuarter = 3;
// row parts of the fused spline adjoint's per-tile bias-gradient sums
constexpr int kSplineBwdRowParts = 3;

// The next coupling layer's ScalarAffine, applied by layer l's fused spline
// kernel on its way out (n_dim even): th_next = that layer's parameters (scale,
// shift first), cond16 [M, ldc16] = its bf16 conditioning operand
struct SplineFold {
  const float* th_next;
  uint16_t* cond16;
  int ldc16;
};

// the last Linear of layer l fused with the spline (tc_spline.cu); ldp holds
// up to kSplineEpiPerQuarter * n_groups partials per row (partial-major,
// [parts, M]; one per group when the kernel stages x in boxes), which are
// then added to ld. With fold, *folded says whether the kernel applied the
// next layer's affine (and added its log-determinant to ld after this
// layer's): only the x-box path does; otherwise the caller applies it.
// With ld == nullptr the partials stay in ldp for the caller to add later
// (ld_reduce_steps); *parts_out gets their count.
int tc_linear_spline(cudaStream_t st, const FlowGeom& g, const FmcFlow* f, int l, const uint16_t* A, int64_t M,
                     int64_t rows_a, bool inverse, float* xa, float* ld, float* ldp,
                     const SplineFold* fold = nullptr, bool* folded = nullptr, int* parts_out = nullptr);

// The log-det partials of up to kLdMaxSteps consecutive fused spline launches
// of one flow pass, left in place and added to ld by one launch: step k's
// parts[k] partials start at ldp + off[k] (partial j of row r at
// off[k] + j * m + r), followed, where th_next[k] is set, by the folded next
// layer's affine log-determinant -- the additions, in order, of one
// per-layer reduction after each launch.
constexpr int kLdMaxSteps = 16;
struct LdSteps {
  int n;
  int parts[kLdMaxSteps];
  int64_t off[kLdMaxSteps];
  const float* th_next[kLdMaxSteps];
};
int ld_reduce_steps(cudaStream_t st, const float* ldp, const LdSteps& s, int64_t m, float* ld, int d, bool inverse);

// adjoint of layer l's last Linear + spline (tc_spline.cu), recomputing the
// Linear from A: dL/dx into gxa (every coordinate), dL/draw in bf16 into graw
// [>= M, ldg] in the padded layout (coordinate t at columns [t * spl_opc,
// t * spl_opc + P), zeros up to (t + 1) * spl_opc; columns past draw_cols(l)
// are not written), and column sums of dL/draw per 128-row tile and row part
// into bpart [ceil(M / 128) * kSplineBwdRowParts, nt * P]
int tc_linear_spline_bwd(cudaStream_t st, const FlowGeom& g, const FmcFlow* f, int l, const uint16_t* A, int64_t M,
                         int64_t rows_a, const float* xa, const float* gy, float gld, float* gxa, uint16_t* graw,
                         int64_t ldg, float* bpart);

// theta (fp32, packed) -> zero-padded bf16 weight segments (FlowGeom::w16_off)
// and their transposes (FlowGeom::w16t_off)
int pack_bf16_weights(const FlowGeom& g, const float* theta, uint16_t* w16, cudaStream_t st);

// whether tc_gemm writes a bf16 output through TMA stores (and so can leave
// EpiArgs::colpart column sums): 16-byte aligned rows, one 64 x 32 box
bool tc_gemm_stages_output(const void* C, int64_t ldc, int n_store, int64_t M);

// C = epi(A . B^T) on tcgen05; A [rows_a, K] bf16 (K a multiple of 64, rows_a
// a multiple of 128 covering M), B [rows_b, K] bf16 (rows_b a multiple of 256
// covering N). bf16 epilogues store n_store columns (zeros beyond N), fp32
// epilogues n_store (= N) columns.
// bn: the output tile width, 128 or 256 (0: 256 when N > 128, else 128);
// pair: 256-row tiles on CTA pairs (cta_group::2) where the epilogue writes
// bf16 through TMA stores and the tile is 256 columns wide
int tc_gemm(cudaStream_t st, const uint16_t* A, int64_t M, int64_t rows_a, int K, const uint16_t* B, int N,
            int rows_b, const tc::EpiArgs& ep, void* C, int64_t ldc, int n_store, int epi, int bn = 0,
            bool pair = false, int64_t lda = 0, int stages = 0);

// scratch (floats) that tc_gemm's fp32 mode uses for split-K partials of an
// M x N x K product when EpiArgs::kpart is given (0: it would not split)
size_t splitk_scratch_floats(int64_t M, int N, int K, int kslices = 0);

// weight gradient C[out, in] = sum over n rows of G[r, out] * X[r, in] on the
// tensor cores, both operands read MN-major from their row-major bf16 buffers
// (gemm_tc.cu)
int tc_gemm_wgrad(cudaStream_t st, const uint16_t* G, int64_t ldg, int out, const uint16_t* X, int64_t ldx, int in,
                  int64_t n, const tc::EpiArgs& ep, float* C, int64_t ldc);

}  // namespace fmc
