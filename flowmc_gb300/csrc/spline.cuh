// spline.cuh -- rational-quadratic spline (forward, inverse, adjoint) for one
// coordinate, templated on the bin count K.
//
// Follows flowMC's rqSpline.py:
//   knots     _normalize_bin_sizes / _normalize_knot_slopes / get_params  (:20-39, :310-338)
//   forward   _rational_quadratic_spline_fwd (:42-128)
//   inverse   _safe_quadratic_root + _rational_quadratic_spline_inv (:131-239)
// The bin is picked with a one-hot predicate loop over compile-time knot
// indices (as the reference does), so every array stays in registers.
// The adjoint is written out by hand: through the spline formula, the
// selected bin's knots, the cumulative sums, the two softmaxes and the
// softplus slopes.
#pragma once
#include <cuda_bf16.h>
#include "common.cuh"

namespace fmc {

struct SplineCfg {
  float rmin, rmax, min_bin, min_slope, slope_offset;
};

template <int K>
struct Knots {
  float xp[K + 1], yp[K + 1], sl[K + 1];
  float pw[K], ph[K];  // softmax probabilities (kept for the adjoint)
};

__device__ __forceinline__ float softplus_f(float a) {
  // jax.nn.softplus = logaddexp(a, 0)
  return fmaxf(a, 0.f) + log1pf(expf(-fabsf(a)));
}

template <int K>
__device__ __forceinline__ void softmax_k(const float* r, float (&p)[K]) {
  float m = r[0];
#pragma unroll
  for (int k = 1; k < K; ++k) m = fmaxf(m, r[k]);
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < K; ++k) {
    p[k] = expf(r[k] - m);
    s += p[k];
  }
#pragma unroll
  for (int k = 0; k < K; ++k) p[k] = p[k] / s;
}

// raw: the 3K+1 conditioner outputs of one coordinate
template <int K>
__device__ __forceinline__ void make_knots(const float* raw, const SplineCfg& c, Knots<K>& kn) {
  const float R = c.rmax - c.rmin;
  const float scale = R - (float)K * c.min_bin;
  softmax_k<K>(raw, kn.pw);
  softmax_k<K>(raw + K, kn.ph);
  float cw = 0.f, ch = 0.f;
  kn.xp[0] = c.rmin;
  kn.yp[0] = c.rmin;
#pragma unroll
  for (int k = 0; k < K - 1; ++k) {
    cw += kn.pw[k] * scale + c.min_bin;
    ch += kn.ph[k] * scale + c.min_bin;
    kn.xp[k + 1] = c.rmin + cw;
    kn.yp[k + 1] = c.rmin + ch;
  }
  kn.xp[K] = c.rmax;
  kn.yp[K] = c.rmax;
#pragma unroll
  for (int k = 0; k <= K; ++k) kn.sl[k] = softplus_f(raw[2 * K + k] + c.slope_offset) + c.min_slope;
}

struct Bin {
  float x0, x1, y0, y1, d0, d1;
  int k;
};

template <int K>
__device__ __forceinline__ Bin select_bin(float v, const float (&pos)[K + 1], const Knots<K>& kn) {
  Bin b{kn.xp[0], kn.xp[1], kn.yp[0], kn.yp[1], kn.sl[0], kn.sl[1], 0};
#pragma unroll
  for (int k = 1; k < K; ++k) {
    if (v >= pos[k] && v < pos[k + 1]) b = Bin{kn.xp[k], kn.xp[k + 1], kn.yp[k], kn.yp[k + 1], kn.sl[k], kn.sl[k + 1], k};
  }
  return b;  // bin 0 also covers "no bin" (rqSpline.py:70-72)
}

template <int K>
__device__ __forceinline__ void rqs_fwd(float x, const Knots<K>& kn, float& y, float& ld) {
  const bool below = x <= kn.xp[0];
  const bool above = x >= kn.xp[K];
  const Bin b = select_bin<K>(x, kn.xp, kn);
  const float w = b.x1 - b.x0, h = b.y1 - b.y0;
  const float s = h / w;
  float z = (x - b.x0) / w;
  z = fminf(fmaxf(z, 0.f), 1.f);
  const float sq = z * z;
  const float q = z - sq;
  const float om = 1.f - z;
  const float sq1 = om * om;
  const float st = b.d1 + b.d0 - 2.f * s;
  const float num = h * (s * sq + b.d0 * q);
  const float den = s + st * q;
  y = b.y0 + num / den;
  ld = 2.f * logf(s) + logf(b.d1 * sq + 2.f * s * q + b.d0 * sq1) - 2.f * logf(den);
  if (below) { y = (x - kn.xp[0]) * kn.sl[0] + kn.yp[0]; ld = logf(kn.sl[0]); }
  if (above) { y = (x - kn.xp[K]) * kn.sl[K] + kn.yp[K]; ld = logf(kn.sl[K]); }
}

template <int K>
__device__ __forceinline__ void rqs_inv(float y, const Knots<K>& kn, float& x, float& ld) {
  const bool below = y <= kn.yp[0];
  const bool above = y >= kn.yp[K];
  const Bin b = select_bin<K>(y, kn.yp, kn);
  const float w = b.x1 - b.x0, h = b.y1 - b.y0;
  const float s = h / w;
  float ww = (y - b.y0) / h;
  ww = fminf(fmaxf(ww, 0.f), 1.f);
  const float st = b.d1 + b.d0 - 2.f * s;
  const float c = -s * ww;
  const float bb = b.d0 - st * ww;
  const float a = s - bb;
  // _safe_quadratic_root (rqSpline.py:131-155)
  const float disc = bb * bb - 4.f * a * c;
  float sqd = sqrtf(fmaxf(disc, 1.17549435e-38f));
  if (!(disc > 0.f)) sqd = 0.f;
  const float num = (bb >= 0.f) ? 2.f * c : -bb + sqd;
  const float dnm = (bb >= 0.f) ? -bb - sqd : 2.f * a;
  float z = num / dnm;
  z = fminf(fmaxf(z, 0.f), 1.f);
  x = w * z + b.x0;
  const float sq = z * z;
  const float q = z - sq;
  const float om = 1.f - z;
  const float sq1 = om * om;
  const float den = s + st * q;
  ld = -2.f * logf(s) - logf(b.d1 * sq + 2.f * s * q + b.d0 * sq1) + 2.f * logf(den);
  if (below) { x = (y - kn.yp[0]) / kn.sl[0] + kn.xp[0]; ld = -logf(kn.sl[0]); }
  if (above) { x = (y - kn.yp[K]) / kn.sl[K] + kn.xp[K]; ld = -logf(kn.sl[K]); }
}

// Adjoint of (y, ld) = rqs_fwd(x; raw): given gy = dL/dy and gl = dL/dld,
// returns dL/dx and accumulates dL/draw[0..3K] into graw.
template <int K>
__device__ __forceinline__ float rqs_fwd_adjoint(float x, const float* raw, const SplineCfg& c, const Knots<K>& kn,
                                                 float gy, float gl, float* graw) {
  float gX[K + 1], gY[K + 1], gD[K + 1];
#pragma unroll
  for (int k = 0; k <= K; ++k) { gX[k] = 0.f; gY[k] = 0.f; gD[k] = 0.f; }
  float gx = 0.f;
  const bool below = x <= kn.xp[0];
  const bool above = x >= kn.xp[K];
  if (below) {
    gx = gy * kn.sl[0];
    gD[0] = gy * (x - kn.xp[0]) + gl / kn.sl[0];
  } else if (above) {
    gx = gy * kn.sl[K];
    gD[K] = gy * (x - kn.xp[K]) + gl / kn.sl[K];
  } else {
    const Bin b = select_bin<K>(x, kn.xp, kn);
    const float w = b.x1 - b.x0, h = b.y1 - b.y0;
    const float s = h / w;
    const float zr = (x - b.x0) / w;
    const float z = fminf(fmaxf(zr, 0.f), 1.f);
    const float sq = z * z, q = z - sq, om = 1.f - z, sq1 = om * om;
    const float st = b.d1 + b.d0 - 2.f * s;
    const float num = h * (s * sq + b.d0 * q);
    const float den = s + st * q;
    const float A = b.d1 * sq + 2.f * s * q + b.d0 * sq1;
    // y = y0 + num/den ; ld = 2 log s + log A - 2 log den
    const float g_num = gy / den;
    const float g_den = -gy * num / (den * den) - 2.f * gl / den;
    const float g_A = gl / A;
    float g_s = 2.f * gl / s;
    float g_h = g_num * (s * sq + b.d0 * q);
    g_s += g_num * h * sq;
    float g_sq = g_num * h * s;
    float g_d0 = g_num * h * q;
    float g_q = g_num * h * b.d0;
    // den = s + (d1 + d0 - 2 s) q
    g_s += g_den * (1.f - 2.f * q);
    float g_d1 = g_den * q;
    g_d0 += g_den * q;
    g_q += g_den * st;
    // A = d1 sq + 2 s q + d0 (1-z)^2
    g_d1 += g_A * sq;
    g_sq += g_A * b.d1;
    g_s += g_A * 2.f * q;
    g_q += g_A * 2.f * s;
    g_d0 += g_A * sq1;
    float g_z = -g_A * b.d0 * 2.f * om;
    // q = z - z^2, sq = z^2
    g_z += g_q * (1.f - 2.f * z) + g_sq * 2.f * z;
    const float g_zr = (zr > 0.f && zr < 1.f) ? g_z : 0.f;
    // zr = (x - x0)/w ; s = h/w
    gx = g_zr / w;
    float g_x0 = -g_zr / w;
    float g_w = -g_zr * zr / w - g_s * s / w;
    g_h += g_s / w;
    // w = x1 - x0, h = y1 - y0
    const float g_x1 = g_w;
    g_x0 -= g_w;
    const float g_y1 = g_h;
    const float g_y0 = gy - g_h;
#pragma unroll
    for (int k = 0; k < K; ++k) {
      if (k == b.k) {
        gX[k] += g_x0; gX[k + 1] += g_x1;
        gY[k] += g_y0; gY[k + 1] += g_y1;
        gD[k] += g_d0; gD[k + 1] += g_d1;
      }
    }
  }
  // knots: X_k = rmin + sum_{i<k} w_i for 1 <= k <= K-1 (X_0, X_K constant)
  const float scale = (c.rmax - c.rmin) - (float)K * c.min_bin;
  float gpw[K], gph[K];
  float accx = 0.f, accy = 0.f;
#pragma unroll
  for (int i = K - 1; i >= 0; --i) {
    // g_w[i] = sum_{k=i+1}^{K-1} gX[k]
    gpw[i] = accx * scale;
    gph[i] = accy * scale;
    if (i >= 1) { accx += gX[i]; accy += gY[i]; }
  }
  // softmax adjoint
  float dw = 0.f, dh = 0.f;
#pragma unroll
  for (int i = 0; i < K; ++i) { dw += kn.pw[i] * gpw[i]; dh += kn.ph[i] * gph[i]; }
#pragma unroll
  for (int i = 0; i < K; ++i) {
    graw[i] = kn.pw[i] * (gpw[i] - dw);
    graw[K + i] = kn.ph[i] * (gph[i] - dh);
  }
  // slopes: d_k = softplus(raw + off) + min_slope -> sigmoid
#pragma unroll
  for (int k = 0; k <= K; ++k) {
    const float a = raw[2 * K + k] + c.slope_offset;
    const float sg = 1.f / (1.f + expf(-a));
    graw[2 * K + k] = gD[k] * sg;
  }
  return gx;
}

// ---------------------------------------------------------------- inference, one bin
// Inference-only spline for the BF16 path: the same function as make_knots +
// rqs_fwd / rqs_inv, but only the bin that holds v is built. Both softmax
// normalisers are still needed (every knot depends on them), the knot
// positions are running sums whose last value at or below v picks the bin
// (identical to the one-hot selection: knots increase, so exactly one k has
// knot_k <= v < knot_{k+1}), and only that bin's two slopes go through the
// softplus. Exponentials, logarithms and divisions use the fast hardware
// approximations; with bf16 conditioner weights their error is far below the
// inputs' own rounding. raw: the 3K+1 conditioner outputs with bias added.
// log(1 + e) with e = exp(-|a|) <= 1 as __logf(1 + e): where 1 + e rounds
// to 1 the error is at most e < 2^-24 in absolute terms, far below the
// minimum knot slope (1e-4) the result is added to
__device__ __forceinline__ float softplus_fast(float a) {
  return fmaxf(a, 0.f) + __logf(1.f + __expf(-fabsf(a)));
}

// 2^x on the SFU (ex2.approx.ftz.f32); softmax arguments are <= 0 after the
// max subtraction, so the approximation's relative error bounds the result
__device__ __forceinline__ float ex2_approx(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// Packed FP32 pairs (f32x2: two lanes of a 64-bit register pair per
// instruction) and the three-input maximum, both sm_100-family instructions.
__device__ __forceinline__ float fmax3(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
__device__ __forceinline__ uint64_t f2_pack(float lo, float hi) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
  return r;
}
__device__ __forceinline__ void f2_unpack(uint64_t v, float& lo, float& hi) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ uint64_t f2_fma(uint64_t a, uint64_t b, uint64_t c) {
  uint64_t d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ uint64_t f2_add(uint64_t a, uint64_t b) {
  uint64_t d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
// a[i] += b[i] for i < N, adjacent pairs as one f32x2 add
template <int N>
__device__ __forceinline__ void add_f2(float* a, const float* b) {
#pragma unroll
  for (int i = 0; i + 1 < N; i += 2) f2_unpack(f2_add(f2_pack(a[i], a[i + 1]), f2_pack(b[i], b[i + 1])), a[i], a[i + 1]);
  if (N & 1) a[N - 1] += b[N - 1];
}

// Unnormalised softmax weights of the K bin widths and K bin heights,
// ew[k] = e^(raw[k] - max) as one FFMA + ex2 each, and their sums. The
// FFMAs and the sums run on adjacent pairs as f32x2 (the sums as two
// interleaved partial sums, added at the end).
template <int K>
__device__ __forceinline__ void softmax_weights(const float (&raw)[3 * K + 1], float (&ew)[K], float (&eh)[K],
                                                float& sw, float& sh) {
  constexpr float kLog2e = 1.4426950408889634f;
  float mw = raw[0], mh = raw[K];
#pragma unroll
  for (int k = 1; k < K; k += 2) {
    if (k + 1 < K) {
      mw = fmax3(mw, raw[k], raw[k + 1]);
      mh = fmax3(mh, raw[K + k], raw[K + k + 1]);
    } else {
      mw = fmaxf(mw, raw[k]);
      mh = fmaxf(mh, raw[K + k]);
    }
  }
  const float nmw = -mw * kLog2e, nmh = -mh * kLog2e;
  const uint64_t l2 = f2_pack(kLog2e, kLog2e), nw2 = f2_pack(nmw, nmw), nh2 = f2_pack(nmh, nmh);
  uint64_t sw2 = f2_pack(0.f, 0.f), sh2 = sw2;
#pragma unroll
  for (int k = 0; k + 1 < K; k += 2) {
    float a0, a1, b0, b1;
    f2_unpack(f2_fma(f2_pack(raw[k], raw[k + 1]), l2, nw2), a0, a1);
    f2_unpack(f2_fma(f2_pack(raw[K + k], raw[K + k + 1]), l2, nh2), b0, b1);
    ew[k] = ex2_approx(a0);
    ew[k + 1] = ex2_approx(a1);
    eh[k] = ex2_approx(b0);
    eh[k + 1] = ex2_approx(b1);
    sw2 = f2_add(sw2, f2_pack(ew[k], ew[k + 1]));
    sh2 = f2_add(sh2, f2_pack(eh[k], eh[k + 1]));
  }
  float a, b;
  f2_unpack(sw2, a, b);
  sw = a + b;
  f2_unpack(sh2, a, b);
  sh = a + b;
  if (K & 1) {
    ew[K - 1] = ex2_approx(fmaf(raw[K - 1], kLog2e, nmw));
    eh[K - 1] = ex2_approx(fmaf(raw[2 * K - 1], kLog2e, nmh));
    sw += ew[K - 1];
    sh += eh[K - 1];
  }
}

// The spline of the bin that holds v only, for the fused tensor-core
// epilogue (same function as rqs_forward/rqs_inverse up to rounding):
// unnormalised softmax weights (softmax_weights), the bin
// found by comparing v with the running knots while carrying only what the
// bin needs (cumulative sums before it, its own weights, its two slope
// parameters), and one log for the log-determinant.
template <int K, bool INV>
__device__ __forceinline__ void rqs_apply_fast(const float (&raw)[3 * K + 1], float v, const SplineCfg& c, float& out,
                                               float& ld) {
  float ew[K], eh[K], sw, sh;
  softmax_weights<K>(raw, ew, eh, sw, sh);
  const float scale = (c.rmax - c.rmin) - (float)K * c.min_bin;
  const float isw = __fdividef(1.f, sw), ish = __fdividef(1.f, sh), iscale = __fdividef(1.f, scale);
  const float fw = scale * isw, fh = scale * ish;   // knot spacing per unit of softmax weight
  // knot k = rmin + f * (sum_{j<k} e_j + k * min_bin / f) = rmin + f * (sum_{j<k} e'_j)
  // with e'_j = e_j + min_bin / f: the bin is found by comparing the running
  // sums of e' with (v - rmin) / f (no per-knot multiply), its left knots are
  // rmin + f * (the sums before it) and its width and height f * e'_bin. Bin 0
  // by default (also covers v below the range).
  const float dw = c.min_bin * sw * iscale, dh = c.min_bin * sh * iscale;
  float ewp[K], ehp[K];
#pragma unroll
  for (int k = 0; k + 1 < K; k += 2) {
    f2_unpack(f2_add(f2_pack(ew[k], ew[k + 1]), f2_pack(dw, dw)), ewp[k], ewp[k + 1]);
    f2_unpack(f2_add(f2_pack(eh[k], eh[k + 1]), f2_pack(dh, dh)), ehp[k], ehp[k + 1]);
  }
  if (K & 1) {
    ewp[K - 1] = ew[K - 1] + dw;
    ehp[K - 1] = eh[K - 1] + dh;
  }
  const float a = (v - c.rmin) * (INV ? sh : sw) * iscale;
  float cw = 0.f, ch = 0.f, bw = 0.f, bh = 0.f, ebw = ewp[0], ebh = ehp[0];
  float r0 = raw[2 * K], r1 = raw[2 * K + 1];
  bool last = false;   // the bin is the last one, whose right knot is exactly rmax
#pragma unroll
  for (int k = 1; k < K; ++k) {
    cw += ewp[k - 1];
    ch += ehp[k - 1];
    const bool in = (INV ? ch : cw) <= a;
    if (in) {
      bw = cw; bh = ch; ebw = ewp[k]; ebh = ehp[k];
      r0 = raw[2 * K + k];
      r1 = raw[2 * K + k + 1];
    }
    if (k == K - 1) last = in;
  }
  const float x0 = fmaf(bw, fw, c.rmin);
  const float y0 = fmaf(bh, fh, c.rmin);
  const float w = last ? c.rmax - x0 : ebw * fw;
  const float h = last ? c.rmax - y0 : ebh * fh;
  const float d0 = softplus_fast(r0 + c.slope_offset) + c.min_slope;
  const float d1 = softplus_fast(r1 + c.slope_offset) + c.min_slope;
  const float s = __fdividef(h, w);
  const float st = d1 + d0 - 2.f * s;
  float z;
  if (!INV) {
    z = fminf(fmaxf(__fdividef(v - x0, w), 0.f), 1.f);
  } else {
    const float ww = fminf(fmaxf(__fdividef(v - y0, h), 0.f), 1.f);
    const float cq = -s * ww;
    const float bq = d0 - st * ww;
    const float aq = s - bq;
    const float disc = bq * bq - 4.f * aq * cq;
    // the hardware square-root approximation (one instruction), like the
    // other fast approximations of this path
    float sqd = 0.f;
    if (disc > 0.f) asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(sqd) : "f"(disc));
    const float num = (bq >= 0.f) ? 2.f * cq : -bq + sqd;
    const float dnm = (bq >= 0.f) ? -bq - sqd : 2.f * aq;
    z = fminf(fmaxf(__fdividef(num, dnm), 0.f), 1.f);
  }
  const float sq = z * z, q = z - sq, om = 1.f - z;
  const float den = s + st * q;
  const float A = d1 * sq + 2.f * s * q + d0 * om * om;
  // log-det 2 log s + log A - 2 log den as one log; log d0 / log d1 in the tails
  float arg = __fdividef(s * s * A, den * den);
  if (!INV) {
    out = y0 + __fdividef(h * (s * sq + d0 * q), den);
    if (v <= c.rmin) { out = (v - c.rmin) * d0 + c.rmin; arg = d0; }
    if (v >= c.rmax) { out = (v - c.rmax) * d1 + c.rmax; arg = d1; }
    ld = __logf(arg);
  } else {
    out = w * z + x0;
    if (v <= c.rmin) { out = __fdividef(v - c.rmin, d0) + c.rmin; arg = d0; }
    if (v >= c.rmax) { out = __fdividef(v - c.rmax, d1) + c.rmax; arg = d1; }
    ld = -__logf(arg);
  }
}

// Adjoint of rqs_apply_fast<K, false> for the BF16 training path: given
// gy = dL/dy and gl = dL/dlogdet, returns dL/dx and writes dL/draw[0..3K] as
// bf16 to out. Same derivative as rqs_fwd_adjoint, organised around the one
// bin that holds x: only its two knots carry gradient into the cumulative
// widths/heights (so dL/dw_i is a two-term prefix rule) and only its two
// slopes go through the softplus derivative; the rest of the slope
// gradients are exactly zero.
template <int K>
__device__ __forceinline__ float rqs_fwd_adjoint_fast(const float (&raw)[3 * K + 1], float x, float gy, float gl,
                                                      const SplineCfg& c, uint16_t* __restrict__ out) {
  float pw[K], ph[K], sw, sh;
  softmax_weights<K>(raw, pw, ph, sw, sh);
  const float iw = __fdividef(1.f, sw), ih = __fdividef(1.f, sh);
#pragma unroll
  for (int k = 0; k < K; ++k) {
    pw[k] *= iw;
    ph[k] *= ih;
  }
  const float scale = (c.rmax - c.rmin) - (float)K * c.min_bin;
  // the bin: cumulative probabilities before it and its own (see rqs_apply_fast)
  float cpw = 0.f, cph = 0.f, bwn = 0.f, bhn = 0.f, ebw = pw[0], ebh = ph[0];
  float r0 = raw[2 * K], r1 = raw[2 * K + 1];
  int kb = 0;
#pragma unroll
  for (int k = 1; k < K; ++k) {
    cpw += pw[k - 1];
    cph += ph[k - 1];
    if (x >= fmaf(cpw, scale, fmaf((float)k, c.min_bin, c.rmin))) {
      bwn = cpw; bhn = cph; ebw = pw[k]; ebh = ph[k]; kb = k;
      r0 = raw[2 * K + k];
      r1 = raw[2 * K + k + 1];
    }
  }
  const bool last = kb == K - 1;   // the last knot is exactly rmax
  const float x0 = fmaf(bwn, scale, fmaf((float)kb, c.min_bin, c.rmin));
  const float y0 = fmaf(bhn, scale, fmaf((float)kb, c.min_bin, c.rmin));
  const float x1 = last ? c.rmax : x0 + fmaf(ebw, scale, c.min_bin);
  const float y1 = last ? c.rmax : y0 + fmaf(ebh, scale, c.min_bin);
  const float a0 = r0 + c.slope_offset, a1 = r1 + c.slope_offset;
  const float d0 = softplus_fast(a0) + c.min_slope, d1 = softplus_fast(a1) + c.min_slope;
  float gx, g_x0 = 0.f, g_x1 = 0.f, g_y0 = 0.f, g_y1 = 0.f, g_d0 = 0.f, g_d1 = 0.f;
  if (x <= c.rmin) {
    gx = gy * d0;
    g_d0 = gy * (x - c.rmin) + __fdividef(gl, d0);
  } else if (x >= c.rmax) {
    gx = gy * d1;
    g_d1 = gy * (x - c.rmax) + __fdividef(gl, d1);
  } else {
    const float w = x1 - x0, h = y1 - y0;
    const float iwd = __fdividef(1.f, w);
    const float s = h * iwd;
    const float zr = (x - x0) * iwd;
    const float z = fminf(fmaxf(zr, 0.f), 1.f);
    const float sq = z * z, q = z - sq, om = 1.f - z, sq1 = om * om;
    const float st = d1 + d0 - 2.f * s;
    const float num = h * (s * sq + d0 * q);
    const float den = s + st * q;
    const float A = d1 * sq + 2.f * s * q + d0 * sq1;
    const float iden = __fdividef(1.f, den);
    // y = y0 + num/den ; ld = 2 log s + log A - 2 log den
    const float g_num = gy * iden;
    const float g_den = -(gy * num * iden + 2.f * gl) * iden;
    const float g_A = __fdividef(gl, A);
    float g_s = __fdividef(2.f * gl, s);
    float g_h = g_num * (s * sq + d0 * q);
    g_s += g_num * h * sq;
    float g_sq = g_num * h * s;
    g_d0 = g_num * h * q;
    float g_q = g_num * h * d0;
    g_s += g_den * (1.f - 2.f * q);
    g_d1 = g_den * q;
    g_d0 += g_den * q;
    g_q += g_den * st;
    g_d1 += g_A * sq;
    g_sq += g_A * d1;
    g_s += g_A * 2.f * q;
    g_q += g_A * 2.f * s;
    g_d0 += g_A * sq1;
    float g_z = -g_A * d0 * 2.f * om;
    g_z += g_q * (1.f - 2.f * z) + g_sq * 2.f * z;
    const float g_zr = (zr > 0.f && zr < 1.f) ? g_z : 0.f;
    gx = g_zr * iwd;
    const float g_w = -(g_zr * zr + g_s * s) * iwd;
    g_h += g_s * iwd;
    g_x0 = -g_zr * iwd - g_w;
    g_x1 = g_w;
    g_y1 = g_h;
    g_y0 = gy - g_h;
  }
  // interior knot k (1 <= k <= K-1) is rmin + sum_{i<k} width_i: dL/dwidth_i
  // collects the gradients of the bin's two knots that lie beyond i, i.e.
  // scale (ax0 + ax1) for i < kb, scale ax1 for i = kb, 0 beyond; the softmax
  // adjoint's sum_j p_j g_j is then closed-form in the bin's sums
  const float ax0 = (kb >= 1) ? g_x0 : 0.f, ax1 = (kb + 1 <= K - 1) ? g_x1 : 0.f;
  const float ay0 = (kb >= 1) ? g_y0 : 0.f, ay1 = (kb + 1 <= K - 1) ? g_y1 : 0.f;
  const float gw_lt = scale * (ax0 + ax1), gw_eq = scale * ax1;
  const float gh_lt = scale * (ay0 + ay1), gh_eq = scale * ay1;
  const float dw = gw_lt * bwn + gw_eq * ebw, dh = gh_lt * bhn + gh_eq * ebh;
#pragma unroll
  for (int i = 0; i < K; ++i) {
    const float gwi = (i < kb) ? gw_lt : ((i == kb) ? gw_eq : 0.f);
    const float ghi = (i < kb) ? gh_lt : ((i == kb) ? gh_eq : 0.f);
    out[i] = __bfloat16_as_ushort(__float2bfloat16_rn(pw[i] * (gwi - dw)));
    out[K + i] = __bfloat16_as_ushort(__float2bfloat16_rn(ph[i] * (ghi - dh)));
  }
  // slopes: d = softplus(raw + offset) + min_slope, d' = sigmoid(raw + offset)
  const float gs0 = g_d0 * __fdividef(1.f, 1.f + __expf(-a0));
  const float gs1 = g_d1 * __fdividef(1.f, 1.f + __expf(-a1));
#pragma unroll
  for (int k = 0; k <= K; ++k) {
    const float v = (k == kb ? gs0 : 0.f) + (k == kb + 1 ? gs1 : 0.f);
    out[2 * K + k] = __bfloat16_as_ushort(__float2bfloat16_rn(v));
  }
  return gx;
}

}  // namespace fmc
