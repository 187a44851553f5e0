// gemm_tc.cu -- host side of the tcgen05 GEMM (tc_gemm.cuh) and the BF16
// conditioner path of the flow: TMA tensor maps, the bf16 weight packing and
// the conditioner MLP as a chain of tensor-core GEMMs with fused epilogues.
#include <cudaTypedefs.h>
#include <cstring>
#include <mutex>
#include "gemm_tc.cuh"
#include "tc_gemm.cuh"

namespace fmc {

__device__ int g_tc_error = 0;   // set by a tcgen05 kernel whose bounded wait expired

// device address of g_tc_error (kernels of other files get it through this)
int tc_error_word(int** out) {
  FMC_CUDA_TRY(cudaGetSymbolAddress((void**)out, g_tc_error));
  return FMC_OK;
}

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  });
  return fn;
}

// 2-D bf16 tensor [outer, inner] with row stride ld (elements), box {64, box_outer}, 128B swizzle
int make_tma_map_bf16(CUtensorMap* m, const void* base, int64_t inner, int64_t outer, int64_t ld, int box_outer);
static int make_map(CUtensorMap* m, const void* base, int64_t inner, int64_t outer, int64_t ld, int box_outer) {
  return make_tma_map_bf16(m, base, inner, outer, ld, box_outer);
}
int make_tma_map_bf16(CUtensorMap* m, const void* base, int64_t inner, int64_t outer, int64_t ld, int box_outer) {
  auto fn = encode_fn();
  FMC_CHECK_SUPPORTED(fn != nullptr, "cuTensorMapEncodeTiled is unavailable");
  FMC_CHECK_ARG(((uintptr_t)base & 15) == 0, "TMA base address must be 16-byte aligned");
  FMC_CHECK_ARG((ld * 2) % 16 == 0, "TMA row stride must be a multiple of 16 bytes");
  FMC_CHECK_ARG(inner >= tc::BK && outer >= box_outer, "tensor smaller than one TMA box");
  cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)outer};
  cuuint64_t strides[1] = {(cuuint64_t)(ld * 2)};
  cuuint32_t box[2] = {(cuuint32_t)tc::BK, (cuuint32_t)box_outer};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled failed (%d): inner=%lld outer=%lld ld=%lld box=%d", (int)r, (long long)inner,
              (long long)outer, (long long)ld, box_outer);
    return FMC_ERR_CUDA;
  }
  return FMC_OK;
}

// The same bf16 tensor [outer, inner] (row stride ld) viewed in 3-D as
// {64 columns, outer rows, inner / 64 chunks}, the chunk stride 128 bytes:
// one box {64, box_outer, ch} lands as ch consecutive [box_outer][128 B]
// K chunks of 128-byte swizzle, the layout of ch one-chunk boxes. inner must
// be a multiple of 64 (no zero fill along K: a ragged last chunk would read
// into the next row).
int make_tma_map_bf16_chunks(CUtensorMap* m, const void* base, int64_t inner, int64_t outer, int64_t ld,
                             int box_outer, int ch) {
  auto fn = encode_fn();
  FMC_CHECK_SUPPORTED(fn != nullptr, "cuTensorMapEncodeTiled is unavailable");
  FMC_CHECK_ARG(((uintptr_t)base & 15) == 0, "TMA base address must be 16-byte aligned");
  FMC_CHECK_ARG((ld * 2) % 16 == 0, "TMA row stride must be a multiple of 16 bytes");
  FMC_CHECK_ARG(inner % tc::BK == 0 && inner / tc::BK >= ch && ch >= 1 && ch <= 8 && ld >= inner,
                "chunked TMA map: K must be a multiple of 64 holding the box's chunks");
  FMC_CHECK_ARG(outer >= box_outer && box_outer <= 256, "tensor smaller than one TMA box");
  cuuint64_t dims[3] = {(cuuint64_t)tc::BK, (cuuint64_t)outer, (cuuint64_t)(inner / tc::BK)};
  cuuint64_t strides[2] = {(cuuint64_t)(ld * 2), (cuuint64_t)(tc::BK * 2)};
  cuuint32_t box[3] = {(cuuint32_t)tc::BK, (cuuint32_t)box_outer, (cuuint32_t)ch};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled (3-D chunks) failed (%d): inner=%lld outer=%lld ld=%lld box=%dx%d", (int)r,
              (long long)inner, (long long)outer, (long long)ld, box_outer, ch);
    return FMC_ERR_CUDA;
  }
  return FMC_OK;
}

// 2-D bf16 tensor [outer, inner] with row stride ld (elements), box
// {box_inner, box_outer}, swizzle 0 / 32 / 64 / 128 bytes (box_inner * 2
// bytes at most the swizzle span), out-of-range elements zero / clipped
int make_tma_map_bf16_box(CUtensorMap* m, const void* base, int64_t inner, int64_t outer, int64_t ld, int box_inner,
                          int box_outer, int swizzle) {
  auto fn = encode_fn();
  FMC_CHECK_SUPPORTED(fn != nullptr, "cuTensorMapEncodeTiled is unavailable");
  FMC_CHECK_ARG(((uintptr_t)base & 15) == 0, "TMA base address must be 16-byte aligned");
  FMC_CHECK_ARG((ld * 2) % 16 == 0, "TMA row stride must be a multiple of 16 bytes");
  FMC_CHECK_ARG((box_inner * 2) % 16 == 0 && box_inner <= 256 && box_outer <= 256, "bad TMA box");
  FMC_CHECK_ARG(swizzle == 0 || box_inner * 2 <= swizzle, "box wider than the swizzle span");
  FMC_CHECK_ARG(inner >= box_inner && outer >= 1, "tensor narrower than one TMA box");
  const CUtensorMapSwizzle sw = swizzle == 32    ? CU_TENSOR_MAP_SWIZZLE_32B
                                : swizzle == 64  ? CU_TENSOR_MAP_SWIZZLE_64B
                                : swizzle == 128 ? CU_TENSOR_MAP_SWIZZLE_128B
                                                 : CU_TENSOR_MAP_SWIZZLE_NONE;
  cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)outer};
  cuuint64_t strides[1] = {(cuuint64_t)(ld * 2)};
  cuuint32_t box[2] = {(cuuint32_t)box_inner, (cuuint32_t)box_outer};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, sw, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled (bf16 box) failed (%d): inner=%lld outer=%lld box=%dx%d swizzle=%d", (int)r,
              (long long)inner, (long long)outer, box_inner, box_outer, swizzle);
    return FMC_ERR_CUDA;
  }
  return FMC_OK;
}

// 2-D fp32 tensor [outer, inner] (row stride = inner elements), box
// {box_inner, box_outer}, no swizzle, out-of-range elements read as zero
int make_tma_map_f32(CUtensorMap* m, const void* base, int64_t inner, int64_t outer, int box_inner, int box_outer) {
  auto fn = encode_fn();
  FMC_CHECK_SUPPORTED(fn != nullptr, "cuTensorMapEncodeTiled is unavailable");
  FMC_CHECK_ARG(((uintptr_t)base & 15) == 0, "TMA base address must be 16-byte aligned");
  FMC_CHECK_ARG((inner * 4) % 16 == 0, "TMA row stride must be a multiple of 16 bytes");
  FMC_CHECK_ARG((box_inner * 4) % 16 == 0 && box_inner <= 256 && box_outer <= 256, "bad TMA box");
  FMC_CHECK_ARG(inner >= box_inner && outer >= 1, "tensor narrower than one TMA box");
  cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)outer};
  cuuint64_t strides[1] = {(cuuint64_t)(inner * 4)};
  cuuint32_t box[2] = {(cuuint32_t)box_inner, (cuuint32_t)box_outer};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<void*>(base), dims, strides, box, estr,
                  CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) {
    set_error("cuTensorMapEncodeTiled (fp32) failed (%d): inner=%lld outer=%lld box=%dx%d", (int)r,
              (long long)inner, (long long)outer, box_inner, box_outer);
    return FMC_ERR_CUDA;
  }
  return FMC_OK;
}

// C[m', n] = sum over the split-K slices of part[s * stride + m * ldc + n]
// (fixed order), m' = m or its image under the row map (rmap_grp > 0: row m
// goes to (m / grp) * keep + m % grp, dropped when m % grp >= keep)
__global__ void k_splitk_reduce(const float* __restrict__ part, int splits, int64_t stride, int64_t M, int n_store,
                                int64_t ldc, float* __restrict__ C, int rmap_grp, int rmap_keep) {
  const int64_t tot = M * n_store;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t m = e / n_store, n = e - m * n_store;
    int64_t mo = m;
    if (rmap_grp > 0) {
      const int64_t t = m / rmap_grp, p = m - t * rmap_grp;
      if (p >= rmap_keep) continue;
      mo = t * rmap_keep + p;
    }
    const int64_t o = m * ldc + n;
    float v = 0.f;
    for (int s = 0; s < splits; ++s) v += part[s * stride + o];
    C[mo * ldc + n] = v;
  }
}

// K-slices for an fp32 GEMM whose tile grid would leave SMs idle: enough to
// fill the SMs, at most 32, at least 4 K-chunks each, never an empty slice
// kslices > 0 asks for that many (at most 32, each at least one K chunk)
static int splitk_count(int64_t tiles, int K, int kslices = 0) {
  const int nk = K / tc::BK;
  int64_t s;
  if (kslices > 0) {
    s = kslices < nk ? kslices : nk;
    if (s > 32) s = 32;
  } else {
    s = sm_count() / (tiles > 0 ? tiles : 1);
    if (s > 32) s = 32;
    if (s > nk / 4) s = nk / 4;
  }
  if (s < 2) return 1;
  const int nks = (nk + (int)s - 1) / (int)s;
  return (nk + nks - 1) / nks;
}

size_t splitk_scratch_floats(int64_t M, int N, int K, int kslices) {
  const int BN = (N > 128) ? 256 : 128;
  const int64_t tiles = (M + tc::BM - 1) / tc::BM * ((N + BN - 1) / BN);
  const int s = splitk_count(tiles, K, kslices);
  return s > 1 ? (size_t)s * (size_t)M * (size_t)N : 0;
}

template <int BN, int STAGES, int EPI, bool TSTORE, int NSTG = 2, int OPM = 0>
static int launch_tc(cudaStream_t st, const CUtensorMap& ma, const CUtensorMap& mb, const CUtensorMap& mc, int64_t M,
                     int N, int K, const tc::EpiArgs& ep, void* C, int64_t ldc, int n_store) {
  using S = tc::Smem<BN, STAGES>;
  // ring + alignment slack + barrier block (1024 with TSTORE, so the staging stays 1024-aligned) + staging
  constexpr int TOTAL = TSTORE ? S::TOTAL + 768 + tc::staging_bytes(NSTG) : S::TOTAL;
  // with the static bias slots (NSTG = 2) and the fail-fast word
  static_assert(TOTAL + (NSTG == 2 ? 1024 : 0) + 16 <= 227 * 1024, "tcgen05 GEMM: shared memory over the per-CTA limit");
  auto kern = tc::k_tc_gemm<BN, STAGES, EPI, TSTORE, false, NSTG, OPM>;
  static bool attr_set = false;
  if (!attr_set) {
    FMC_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, TOTAL));
    attr_set = true;
  }
  int* err = nullptr;
  FMC_CUDA_TRY(cudaGetSymbolAddress((void**)&err, g_tc_error));
  const int64_t mt = (M + tc::BM - 1) / tc::BM;
  const int64_t tiles = mt * ((n_store + BN - 1) / BN);
  FMC_CHECK_SUPPORTED(tiles < (1ll << 26) && M < (1ll << 31), "GEMM too large (%lld tiles)", (long long)tiles);
  int splits = 1;
  if (EPI == tc::TC_EPI_F32 && ep.kpart != nullptr) {
    splits = splitk_count(tiles, K, ep.kslices);
    if ((int64_t)splits * M * ldc > ep.kpart_floats) splits = 1;
  }
  const int64_t items = tiles * splits;
  const int64_t grid = items < sm_count() ? items : sm_count();   // persistent: one CTA per SM
  void* out = splits > 1 ? (void*)ep.kpart : C;
  {
    const bool bf16_out = EPI == tc::TC_EPI_TANH_BF16 || EPI == tc::TC_EPI_DTANH_BF16;
    const int kid = EPI == tc::TC_EPI_TANH_BF16 ? FMC_KT_TC_GEMM_TANH
                    : EPI == tc::TC_EPI_DTANH_BF16 ? FMC_KT_TC_GEMM_DTANH
                                                   : FMC_KT_TC_GEMM_F32;
    // A and B once, C written (bf16 or fp32), the tanh input read back in mode 2
    const double bytes = (double)M * K * 2 + (double)N * K * 2 + (double)M * N * (bf16_out ? 2 : 4) +
                         (EPI == tc::TC_EPI_DTANH_BF16 ? (double)M * N * 2 : 0.0);
    KernelTimer kt(kid, st, 2.0 * (double)M * N * K, bytes);
    note_grid(kid, (int)grid, 1);
    kern<<<(unsigned)grid, tc::kThreads, TOTAL, st>>>(ma, mb, mc, (int)M, N, K, ep, out, ldc, n_store, splits,
                                                     M * ldc, err);
    FMC_LAUNCH_CHECK();
  }
  if (splits > 1) {
    int64_t blocks = (M * n_store + 255) / 256;
    if (blocks > (int64_t)sm_count() * 8) blocks = (int64_t)sm_count() * 8;
    k_splitk_reduce<<<(int)blocks, 256, 0, st>>>(ep.kpart, splits, M * ldc, M, n_store, ldc, (float*)C, ep.rmap_grp,
                                                ep.rmap_keep);
    FMC_LAUNCH_CHECK();
  }
  return FMC_OK;
}

// the CTA-pair form (bf16 outputs through TMA stores): 256-row tiles, a
// persistent grid of as many clusters of 2 as can be resident
template <int BN, int STAGES, int EPI, int NSTG = 2>
static int launch_tc_pair(cudaStream_t st, const CUtensorMap& ma, const CUtensorMap& mb, const CUtensorMap& mc,
                          int64_t M, int N, int K, const tc::EpiArgs& ep, void* C, int64_t ldc, int n_store) {
  using S = tc::Smem<BN / 2, STAGES>;
  constexpr int TOTAL = S::TOTAL + 768 + tc::staging_bytes(NSTG);
  static_assert(TOTAL + (NSTG == 2 ? 1024 : 0) + 16 <= 227 * 1024, "tcgen05 GEMM: shared memory over the per-CTA limit");
  auto kern = tc::k_tc_gemm<BN, STAGES, EPI, true, true, NSTG>;
  static bool attr_set = false;
  if (!attr_set) {
    FMC_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, TOTAL));
    attr_set = true;
  }
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.blockDim = dim3(tc::kThreads, 1, 1);
  cfg.dynamicSmemBytes = TOTAL;
  cfg.stream = st;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  static int max_pairs = 0;
  if (max_pairs == 0) {
    cfg.gridDim = dim3(2 * (unsigned)(sm_count() / 2), 1, 1);
    int n = 0;
    FMC_CUDA_TRY(cudaOccupancyMaxActiveClusters(&n, (void*)kern, &cfg));
    max_pairs = n > 0 ? n : 1;
  }
  int* err = nullptr;
  FMC_CUDA_TRY(cudaGetSymbolAddress((void**)&err, g_tc_error));
  const int64_t tiles = (M + 2 * tc::BM - 1) / (2 * tc::BM) * ((n_store + BN - 1) / BN);
  FMC_CHECK_SUPPORTED(tiles < (1ll << 26) && M < (1ll << 31), "GEMM too large (%lld tiles)", (long long)tiles);
  const int64_t pairs = tiles < max_pairs ? tiles : max_pairs;
  cfg.gridDim = dim3(2 * (unsigned)pairs, 1, 1);
  const int kid = EPI == tc::TC_EPI_TANH_BF16 ? FMC_KT_TC_GEMM_TANH : FMC_KT_TC_GEMM_DTANH;
  const double bytes = (double)M * K * 2 + (double)N * K * 2 + (double)M * N * 2 +
                       (EPI == tc::TC_EPI_DTANH_BF16 ? (double)M * N * 2 : 0.0);
  KernelTimer kt(kid, st, 2.0 * (double)M * N * K, bytes);
  note_grid(kid, (int)(2 * pairs), 2);
  int Mi = (int)M, one = 1;
  int64_t stride = M * ldc;
  FMC_CUDA_TRY(cudaLaunchKernelEx(&cfg, kern, ma, mb, mc, Mi, N, K, ep, C, ldc, n_store, one, stride, err));
  FMC_LAUNCH_CHECK();
  return FMC_OK;
}

// Weight gradient C[out, in] = sum over the n batch rows of G[r, out] * X[r, in]
// (fp32, split along the batch when the tile grid is small), reading both
// operands MN-major straight from their row-major bf16 buffers: G [n, ldg]
// and X [n, ldx], columns beyond out / in zero up to the pitch (a multiple of
// 64), rows past n read as zeros through the tensor maps (for n < 64 the
// maps cover 64 rows, and rows [n, 64) must hold zeros).
int tc_gemm_wgrad(cudaStream_t st, const uint16_t* G, int64_t ldg, int out, const uint16_t* X, int64_t ldx, int in,
                  int64_t n, const tc::EpiArgs& ep, float* C, int64_t ldc) {
  FMC_CHECK_ARG(ldg % 64 == 0 && ldx % 64 == 0 && ldg >= out && ldx >= in, "operand pitches must cover the outputs "
                "and be multiples of 64");
  FMC_CHECK_ARG(n >= 1 && out >= 1 && in >= 1 && ldc >= in, "bad sizes");
  CUtensorMap ma, mb, mc;
  const int64_t rows = n < 64 ? 64 : n;
  int rc = make_map(&ma, G, ldg, rows, ldg, 64);
  if (rc) return rc;
  const int BN = in > 128 ? 256 : 128;
  if ((rc = make_map(&mb, X, ldx, rows, ldx, 64))) return rc;
  memset(&mc, 0, sizeof(mc));
  const int K = (int)FlowGeom::rup(n, 64);
  FMC_CHECK_SUPPORTED(n < (1ll << 31), "batch too large");
  if (BN == 256) return launch_tc<256, 4, tc::TC_EPI_F32, false, 2, 3>(st, ma, mb, mc, out, in, K, ep, C, ldc, in);
  return launch_tc<128, 4, tc::TC_EPI_F32, false, 2, 3>(st, ma, mb, mc, out, in, K, ep, C, ldc, in);
}

bool tc_gemm_stages_output(const void* C, int64_t ldc, int n_store, int64_t M) {
  return ((uintptr_t)C & 15) == 0 && (ldc * 2) % 16 == 0 && n_store >= 64 && M >= 32;
}

int tc_gemm(cudaStream_t st, const uint16_t* A, int64_t M, int64_t rows_a, int K, const uint16_t* B, int N,
            int rows_b, const tc::EpiArgs& ep, void* C, int64_t ldc, int n_store, int epi, int bn, bool pair,
            int64_t lda, int stages) {
  FMC_CHECK_ARG(K % tc::BK == 0 && K >= tc::BK, "K=%d must be a positive multiple of 64", K);
  FMC_CHECK_ARG(rows_a % tc::BM == 0 && rows_a >= M, "A rows %lld must cover M and be a multiple of 128",
                (long long)rows_a);
  FMC_CHECK_ARG(rows_b % 256 == 0 && rows_b >= N, "B rows %d must cover N and be a multiple of 256", rows_b);
  FMC_CHECK_ARG(n_store <= ldc, "n_store %d > ldc %lld", n_store, (long long)ldc);
  if (epi == tc::TC_EPI_TANH_BF16 || epi == tc::TC_EPI_BIAS_F32) FMC_CHECK_ARG(ep.bias != nullptr, "bias is NULL");
  if (epi == tc::TC_EPI_DTANH_BF16) FMC_CHECK_ARG(ep.aux != nullptr, "aux is NULL");
  if (M <= 0) return FMC_OK;
  const int BN = (bn == 128 || bn == 256) ? bn : ((N > 128) ? 256 : 128);
  CUtensorMap ma, mb, mc;
  FMC_CHECK_ARG(lda == 0 || lda >= K, "lda %lld < K %d", (long long)lda, K);
  int rc = make_map(&ma, A, K, rows_a, lda > 0 ? lda : K, tc::BM);
  if (rc) return rc;
  if ((rc = make_map(&mb, B, K, rows_b, K, BN))) return rc;
  // bf16 outputs go out through TMA stores when C can carry a tensor map
  // (16-byte aligned rows, at least one 64 x 32 box)
  const bool bf16_out = epi == tc::TC_EPI_TANH_BF16 || epi == tc::TC_EPI_DTANH_BF16;
  const bool tstore = bf16_out && tc_gemm_stages_output(C, ldc, n_store, M);
  FMC_CHECK_ARG(ep.colpart == nullptr || (epi == tc::TC_EPI_DTANH_BF16 && tstore),
                "column sums need the tanh-adjoint epilogue with staged TMA stores");
  memset(&mc, 0, sizeof(mc));
  if (tstore && (rc = make_map(&mc, C, n_store, M, ldc, 32))) return rc;
  if (pair && tstore && BN == 256) {
    // B in boxes of half the tile's rows: each CTA of a pair loads one half
    if ((rc = make_map(&mb, B, K, rows_b, K, BN / 2))) return rc;
    // a pair stage holds half the B rows (32 KB with A): six stages and one
    // staging buffer per warp where a tile takes several K blocks (deeper
    // prefetch for the same shared memory), four and two otherwise
    if (K >= 4 * tc::BK) {
      if (epi == tc::TC_EPI_TANH_BF16)
        return launch_tc_pair<256, 6, tc::TC_EPI_TANH_BF16, 1>(st, ma, mb, mc, M, N, K, ep, C, ldc, n_store);
      if (epi == tc::TC_EPI_DTANH_BF16)
        return launch_tc_pair<256, 6, tc::TC_EPI_DTANH_BF16, 1>(st, ma, mb, mc, M, N, K, ep, C, ldc, n_store);
    }
    if (epi == tc::TC_EPI_TANH_BF16)
      return launch_tc_pair<256, 4, tc::TC_EPI_TANH_BF16>(st, ma, mb, mc, M, N, K, ep, C, ldc, n_store);
    if (epi == tc::TC_EPI_DTANH_BF16)
      return launch_tc_pair<256, 4, tc::TC_EPI_DTANH_BF16>(st, ma, mb, mc, M, N, K, ep, C, ldc, n_store);
  }
#define TC_CASE(E)                                                                                            \
  if (epi == E) {                                                                                             \
    if (BN == 256) return launch_tc<256, 4, E, false>(st, ma, mb, mc, M, N, K, ep, C, ldc, n_store);          \
    return launch_tc<128, 4, E, false>(st, ma, mb, mc, M, N, K, ep, C, ldc, n_store);                         \
  }
  // 256-column tiles with staged stores: a four-deep ring and one staging
  // buffer per warp where a tile takes several K blocks (the ring's depth
  // hides the operand loads), three stages and two buffers (and the bias in
  // shared memory) where one or two K blocks make the epilogue the limit
#define TC_CASE_TS(E)                                                                                         \
  if (epi == E && tstore) {                                                                                   \
    if (BN == 256 && K >= 4 * tc::BK && stages != 3)                                                          \
      return launch_tc<256, 4, E, true, 1>(st, ma, mb, mc, M, N, K, ep, C, ldc, n_store);                     \
    if (BN == 256) return launch_tc<256, 3, E, true, 2>(st, ma, mb, mc, M, N, K, ep, C, ldc, n_store);        \
    return launch_tc<128, 4, E, true, 2>(st, ma, mb, mc, M, N, K, ep, C, ldc, n_store);                       \
  }
  TC_CASE_TS(tc::TC_EPI_TANH_BF16)
  TC_CASE_TS(tc::TC_EPI_DTANH_BF16)
  TC_CASE(tc::TC_EPI_TANH_BF16)
  TC_CASE(tc::TC_EPI_BIAS_F32)
  TC_CASE(tc::TC_EPI_DTANH_BF16)
  TC_CASE(tc::TC_EPI_F32)
#undef TC_CASE
#undef TC_CASE_TS
  set_error("unknown epilogue %d", epi);
  return FMC_ERR_INVALID_ARG;
}

// ------------------------------------------------------------------ packing
// source row of W (fp32 [out, in]) for column c of the transposed copy of
// Linear i of layer l: c itself, or for the last Linear the padded d-raw
// column c = t * opc + p (-1 for a padding column)
__device__ __forceinline__ int wt_src_row(const FlowGeom& g, int l, int i, int c, int out) {
  if (i < g.nh) return c < out ? c : -1;
  const int t = c / g.spl_opc, p = c - t * g.spl_opc;
  return (t < g.nt(l) && p < g.P) ? t * g.P + p : -1;
}

// Blocks of 256 threads; blockIdx.y selects the segment: W_i (zero padded,
// one block per row at a time), W_i^T (32 x 32 tiles through shared memory,
// so both the reads of W and the writes of W^T are coalesced) or the
// grouped copy of the last Linear.
__global__ void k_pack_bf16(FlowGeom g, const float* __restrict__ theta, uint16_t* __restrict__ w16) {
  __shared__ float tile[32][33];
  const int nseg = g.L * (g.nh + 1);
  if ((int)blockIdx.y >= 2 * nseg) {
    // grouped copy of layer l's last Linear for the fused spline kernel
    const int l = blockIdx.y - 2 * nseg;
    const int i = g.nh, in = g.lin_in(l, i), nt = g.nt(l);
    const int cols = g.w16_cols(l, i), DG = g.spl_dg, BN = g.spl_bn, PP = g.spl_pp;
    const int rows = g.spl_groups(l) * BN;
    const float* W = theta + g.layer_off[l] + g.lin_w(l, i);
    uint16_t* dst = w16 + g.w16g_off[l];
    for (int r = blockIdx.x; r < rows; r += gridDim.x) {
      const int grp = r / BN, rr = r - grp * BN;
      const int u = rr / PP, p = rr - u * PP;
      const int t = grp * DG + u;
      const bool live = u < DG && p < g.P && t < nt;
      const float* src = W + ((int64_t)t * g.P + p) * in;
      for (int c = threadIdx.x; c < cols; c += blockDim.x)
        dst[(int64_t)r * cols + c] = f32_to_bf16_rn((live && c < in) ? src[c] : 0.f);
    }
    return;
  }
  const int seg = blockIdx.y % nseg;
  const bool tr = blockIdx.y >= nseg;   // second part of the grid writes W^T
  const int l = seg / (g.nh + 1), i = seg % (g.nh + 1);
  const int out = g.lin_out(l, i), in = g.lin_in(l, i);
  const float* W = theta + g.layer_off[l] + g.lin_w(l, i);
  if (!tr) {
    const int rows = g.w16_rows(l, i), cols = g.w16_cols(l, i);
    uint16_t* dst = w16 + g.w16_off[seg];
    for (int r = blockIdx.x; r < rows; r += gridDim.x)
      for (int c = threadIdx.x; c < cols; c += blockDim.x)
        dst[(int64_t)r * cols + c] = f32_to_bf16_rn((r < out && c < in) ? W[(int64_t)r * in + c] : 0.f);
    return;
  }
  // W^T [rows = round_up(in, 256), cols]: element (r, c) = W[src(c), r]
  const int rows = g.w16t_rows(l, i), cols = g.w16t_cols(l, i);
  uint16_t* dst = w16 + g.w16t_off[seg];
  const int tr_ = (rows + 31) / 32, tc_ = (cols + 31) / 32;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;   // 32 x 8
  for (int tt = blockIdx.x; tt < tr_ * tc_; tt += gridDim.x) {
    const int r0 = (tt / tc_) * 32, c0 = (tt % tc_) * 32;
    // read 32 source rows (columns c0.. of W^T) along r: coalesced
    for (int k = ty; k < 32; k += 8) {
      const int sr = wt_src_row(g, l, i, c0 + k, out);
      const int r = r0 + tx;
      tile[k][tx] = (sr >= 0 && r < in) ? W[(int64_t)sr * in + r] : 0.f;
    }
    __syncthreads();
    for (int k = ty; k < 32; k += 8) {
      const int r = r0 + k, c = c0 + tx;
      if (r < rows && c < cols) dst[(int64_t)r * cols + c] = f32_to_bf16_rn(tile[tx][k]);
    }
    __syncthreads();
  }
}

int pack_bf16_weights(const FlowGeom& g, const float* theta, uint16_t* w16, cudaStream_t st) {
  const int segs = g.L * (g.nh + 1);
  dim3 grid(64, 2 * segs + g.L);
  k_pack_bf16<<<grid, 256, 0, st>>>(g, theta, w16);
  FMC_LAUNCH_CHECK();
  return FMC_OK;
}

// fp32 [m, n] -> bf16 [m, ld] zero padded (ld >= n)
__global__ void k_to_bf16_pad(const float* __restrict__ a, int64_t m, int n, int ld, uint16_t* __restrict__ b) {
  const int64_t tot = m * ld;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < tot; e += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = e / ld;
    const int c = (int)(e - r * ld);
    b[e] = (c < n) ? f32_to_bf16_rn(a[r * n + c]) : (uint16_t)0;
  }
}

int conditioner_bf16_hidden(const FmcFlow* f, const FlowGeom& g, int l, int64_t m, const float* cond,
                            uint16_t* cond16, uint16_t* h16a, uint16_t* h16b, const uint16_t** h_last,
                            cudaStream_t st) {
  const int64_t rows = (m + tc::BM - 1) / tc::BM * tc::BM;
  const int nc = g.nc(l), ncp = g.w16_cols(l, 0);
  if (cond != nullptr) {
    int64_t blocks = (m * ncp + 255) / 256;
    if (blocks > (int64_t)sm_count() * 16) blocks = (int64_t)sm_count() * 16;
    k_to_bf16_pad<<<(int)blocks, 256, 0, st>>>(cond, m, nc, ncp, cond16);
    FMC_LAUNCH_CHECK();
  }
  const float* th = f->theta + g.layer_off[l];
  const uint16_t* a = cond16;
  uint16_t* hbuf[2] = {h16a, h16b};
  for (int i = 0; i < g.nh; ++i) {
    const int seg = l * (g.nh + 1) + i;
    const int K = g.w16_cols(l, i), N = g.lin_out(l, i);
    tc::EpiArgs ep{};
    ep.bias = th + g.lin_b(l, i);
    const int ldo = (int)FlowGeom::rup(N, 64);
    int rc = tc_gemm(st, a, m, rows, K, f->theta_bf16 + g.w16_off[seg], N, g.w16_rows(l, i), ep, hbuf[i & 1], ldo, ldo,
                     tc::TC_EPI_TANH_BF16, f->gemm_bn, f->tile_rows == 256, 0, f->gemm_stages);
    if (rc) return rc;
    a = hbuf[i & 1];
  }
  *h_last = a;
  return FMC_OK;
}

}  // namespace fmc

using namespace fmc;

extern "C" int fmc_tc_gemm_bf16(const uint16_t* A, int64_t M, int64_t rows_a, int32_t K, const uint16_t* B,
                                int32_t N, int32_t rows_b, const float* bias, void* C, int64_t ldc, int32_t n_store,
                                int32_t epilogue, void* stream) {
  FMC_CHECK_ARG(A && B && bias && C, "NULL pointer");
  FMC_CHECK_ARG(epilogue == 0 || epilogue == 1, "epilogue must be 0 (tanh, bf16 out) or 1 (bias, fp32 out)");
  FMC_CHECK_ARG(n_store >= N && n_store <= ldc, "n_store must be in [N, ldc]");
  tc::EpiArgs ep{};
  ep.bias = bias;
  return tc_gemm((cudaStream_t)stream, A, M, rows_a, K, B, N, rows_b, ep, C, ldc, n_store, epilogue);
}

// Failure-path self-test of the bounded waits: one warp initialises an
// mbarrier that nothing will complete and waits on it with mbar_wait (the
// routine every tcgen05 kernel here uses); the wait gives up after about a
// second and the kernel records that it did. Nothing faults or hangs.
__global__ void k_selftest_bounded_wait(int* timed_out) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncwarp();
  if (threadIdx.x == 0) *timed_out = tc::mbar_wait(&bar, 0) ? 0 : 1;
}

__device__ int g_selftest_word = -1;

extern "C" int fmc_selftest_bounded_wait(int32_t* timed_out, void* stream) {
  FMC_CHECK_ARG(timed_out != nullptr, "timed_out is NULL");
  cudaStream_t st = (cudaStream_t)stream;
  int* d = nullptr;
  FMC_CUDA_TRY(cudaGetSymbolAddress((void**)&d, g_selftest_word));
  FMC_CUDA_TRY(cudaMemsetAsync(d, 0xff, sizeof(int), st));
  k_selftest_bounded_wait<<<1, 32, 0, st>>>(d);
  FMC_LAUNCH_CHECK();
  int h = -1;
  FMC_CUDA_TRY(cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost, st));
  FMC_CUDA_TRY(cudaStreamSynchronize(st));
  *timed_out = h;
  return FMC_OK;
}

extern "C" int fmc_device_error_set(int32_t value) {
  FMC_CUDA_TRY(cudaMemcpyToSymbol(g_tc_error, &value, sizeof(int)));
  return FMC_OK;
}

extern "C" int fmc_device_error(int32_t* out, int32_t clear) {
  FMC_CHECK_ARG(out != nullptr, "out is NULL");
  int v = 0;
  FMC_CUDA_TRY(cudaMemcpyFromSymbol(&v, g_tc_error, sizeof(int)));
  if (clear) {
    const int z = 0;
    FMC_CUDA_TRY(cudaMemcpyToSymbol(g_tc_error, &z, sizeof(int)));
  }
  *out = v;
  return FMC_OK;
}
