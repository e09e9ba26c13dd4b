// Shared device helpers: complex arithmetic on double2/float2, cache-hinted
// loads, block reductions in FP64 and the coefficient interpreter.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "qutip_gb300.h"
#include "vern7_tableau.cuh"  // generated from qutip_gb300/vern7_tableau.py

namespace qg {

// ---------------------------------------------------------------- complex --
struct cplx {
  double re, im;
};

__device__ __forceinline__ cplx cmake(double r, double i) { return cplx{r, i}; }
__device__ __forceinline__ cplx cadd(cplx a, cplx b) { return cplx{a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ cplx csub(cplx a, cplx b) { return cplx{a.re - b.re, a.im - b.im}; }
__device__ __forceinline__ cplx cmul(cplx a, cplx b) {
  return cplx{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
__device__ __forceinline__ cplx cscale(cplx a, double s) { return cplx{a.re * s, a.im * s}; }
__device__ __forceinline__ double cabs2(cplx a) { return a.re * a.re + a.im * a.im; }

// Storage element types.  C128 = double2 (16 B), C64 = float2 (8 B).
template <int DT>
struct elem;
template <>
struct elem<QG_C128> {
  using T = double2;
  using R = double;  // accumulation type of the matvec
};
template <>
struct elem<QG_C64> {
  using T = float2;
  using R = float;
};

__device__ __forceinline__ cplx to_c(double2 v) { return cplx{v.x, v.y}; }
__device__ __forceinline__ cplx to_c(float2 v) { return cplx{(double)v.x, (double)v.y}; }
template <typename T>
__device__ __forceinline__ T from_c(cplx v);
template <>
__device__ __forceinline__ double2 from_c<double2>(cplx v) { return make_double2(v.re, v.im); }
template <>
__device__ __forceinline__ float2 from_c<float2>(cplx v) {
  return make_float2((float)v.re, (float)v.im);
}

// Streaming (read-once) loads for operator values and indices: evict-first so
// that the gathered vector keeps its L2 residency.
__device__ __forceinline__ double2 ld_stream(const double2* p) { return __ldcs(p); }
__device__ __forceinline__ float2 ld_stream(const float2* p) { return __ldcs(p); }
__device__ __forceinline__ int ld_stream(const int* p) { return __ldcs(p); }
__device__ __forceinline__ unsigned int ld_stream(const unsigned int* p) { return __ldcs(p); }
__device__ __forceinline__ uint2 ld_stream(const uint2* p) { return __ldcs(p); }
// Gathered vector: read-only path.
__device__ __forceinline__ double2 ld_gather(const double2* p) { return __ldg(p); }
__device__ __forceinline__ float2 ld_gather(const float2* p) { return __ldg(p); }

// ----------------------------------------------- bulk copies, mbarriers --
__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0u;
}
// 1-D bulk copy global -> shared; dst, src and bytes are multiples of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes,
                                         uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// Bounded wait: every thread polls for at most WAIT_CYCLES SM cycles (about a
// second); a block-wide vote decides whether the wait completed.  A wait that
// never completes (it cannot in a correct launch) sets the device fault flag
// instead of hanging the GPU.
constexpr long long WAIT_CYCLES = 2000000000LL;
__device__ __forceinline__ bool mbar_poll(uint64_t* bar, unsigned parity) {
  const long long t0 = clock64();
  bool ok = mbar_try_wait(bar, parity);
  while (!ok && clock64() - t0 < WAIT_CYCLES) ok = mbar_try_wait(bar, parity);
  return ok;
}

// ------------------------------------------------------------ reductions --
// Sum a double over the block; result valid in thread 0.  Fixed order, so the
// result is reproducible for a fixed launch shape.
template <int BLOCK>
__device__ __forceinline__ double block_sum(double v, double* smem /* [BLOCK/32] */) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  if (l == 0) smem[w] = v;
  __syncthreads();
  double r = 0.0;
  if (threadIdx.x < 32) {
    r = (threadIdx.x < BLOCK / 32) ? smem[threadIdx.x] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
  }
  __syncthreads();
  return r;
}

// WRMS term |e|^2 / (atol + rtol sqrt(u))^2 in FP64 (u = |y|^2, e2 = |e|^2) to ~1e-13
// relative without an FP64 square root or division: 1/sqrt(u) and 1/sc start from the FP32
// intrinsics and take one Newton-Raphson step each in FP64 (r <- r (3 - u r^2) / 2 and
// i <- i (2 - sc i), each doubling the correct digits).  An FP64 sqrt and divide cost ~25
// FP64 operations per row, which made the last Vern7 stage the slowest by far on a GPU
// whose FP64 pipe runs at 1/64 of FP32.  Magnitudes below 1e-15 count as zero (their share
// of atol + rtol |y| is below 1e-13 of atol).  Used by the mixed form, whose error estimate
// carries complex64 rounding anyway; the complex128 form keeps IEEE sqrt and division so
// that its step sequence and jump records are the reference's.
__device__ __forceinline__ double wrms_term(double e2, double u, double atol, double rtol) {
  double mag = 0.0;
  if (u > 1e-30) {
    const double r0 = (double)rsqrtf((float)u);
    const double r1 = r0 * fma(-0.5 * u * r0, r0, 1.5);
    mag = u * r1;
  }
  const double sc = fma(rtol, mag, atol);
  const double i0 = (double)__frcp_rn((float)sc);
  const double i1 = i0 * fma(-sc, i0, 2.0);
  return e2 * (i1 * i1);
}

// ---------------------------------------------------- coefficient programs --
// Opcodes shared with qutip_gb300/coefficients.py (OPCODES).
enum : int {
  OP_END = 0, OP_CONST = 1, OP_T = 2, OP_ADD = 3, OP_SUB = 4, OP_MUL = 5, OP_DIV = 6,
  OP_NEG = 7, OP_COS = 8, OP_SIN = 9, OP_EXP = 10, OP_LOG = 11, OP_SQRT = 12, OP_CONJ = 13,
  OP_REAL = 14, OP_IMAG = 15, OP_ABS = 16, OP_POW = 17, OP_COSH = 18, OP_SINH = 19,
  OP_TANH = 20, OP_TAN = 21, OP_ARCTAN = 22, OP_INTERP = 23
};
constexpr int COEF_STACK = 16;

__device__ __forceinline__ cplx c_exp(cplx z) {
  double e = exp(z.re);
  if (z.im == 0.0) return cplx{e, 0.0};
  double s, c;
  sincos(z.im, &s, &c);
  return cplx{e * c, e * s};
}
__device__ __forceinline__ cplx c_log(cplx z) {
  return cplx{log(hypot(z.re, z.im)), atan2(z.im, z.re)};
}
__device__ __forceinline__ cplx c_div(cplx a, cplx b) {
  if (b.im == 0.0) return cplx{a.re / b.re, a.im / b.re};
  double d = b.re * b.re + b.im * b.im;
  return cplx{(a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d};
}
__device__ __forceinline__ cplx c_sqrt(cplx z) {
  if (z.im == 0.0) {
    if (z.re >= 0.0) return cplx{sqrt(z.re), 0.0};
    return cplx{0.0, sqrt(-z.re)};
  }
  // principal branch: sqrt(z) = sqrt((|z|+x)/2) + i sign(y) sqrt((|z|-x)/2)
  double m = hypot(z.re, z.im);
  double r = sqrt(0.5 * (m + z.re));
  double i = sqrt(0.5 * (m - z.re));
  return cplx{r, copysign(i, z.im)};
}
__device__ __forceinline__ cplx c_cos(cplx z) {
  if (z.im == 0.0) return cplx{cos(z.re), 0.0};
  return cplx{cos(z.re) * cosh(z.im), -sin(z.re) * sinh(z.im)};
}
__device__ __forceinline__ cplx c_sin(cplx z) {
  if (z.im == 0.0) return cplx{sin(z.re), 0.0};
  return cplx{sin(z.re) * cosh(z.im), cos(z.re) * sinh(z.im)};
}
__device__ __forceinline__ cplx c_cosh(cplx z) {
  if (z.im == 0.0) return cplx{cosh(z.re), 0.0};
  return cplx{cosh(z.re) * cos(z.im), sinh(z.re) * sin(z.im)};
}
__device__ __forceinline__ cplx c_sinh(cplx z) {
  if (z.im == 0.0) return cplx{sinh(z.re), 0.0};
  return cplx{sinh(z.re) * cos(z.im), cosh(z.re) * sin(z.im)};
}

// Piecewise polynomial table in the constant pool (an interpolated coefficient,
// qutip/core/cy/coefficient.pyx:412-566): consts[k] = (n, order), consts[k+1] =
// (dt, 0), then n breakpoints (real parts), then poly[order+1][n].  Below the first
// breakpoint the value is poly[order][0], from the last one poly[order][n-1];
// inside, the interval is found by dt (uniform breakpoints) or a bisection of at
// most 64 steps, and the polynomial in (t - t_idx) is evaluated by Horner.
__device__ __forceinline__ cplx interp_eval(const double* consts, int k, double t) {
  const int n = (int)consts[2 * k];
  const int order = (int)consts[2 * k + 1];
  const double dt = consts[2 * k + 2];
  const double* tl = consts + 2 * (k + 2);
  const double* poly = consts + 2 * (k + 2 + n);
  if (n <= 0 || order < 0) return cplx{0.0, 0.0};
  const int last = order * n;
  if (t <= tl[0]) return cplx{poly[2 * last], poly[2 * last + 1]};
  if (t >= tl[2 * (n - 1)]) return cplx{poly[2 * (last + n - 1)], poly[2 * (last + n - 1) + 1]};
  long long idx;
  if (dt != 0.0) {
    idx = (long long)((t - tl[0]) / dt);
  } else {
    long long lo = 0, hi = n;
    for (int count = 0; lo + 1 != hi && count < 64; ++count) {
      const long long mid = (lo + hi) / 2;
      if (t < tl[2 * mid]) hi = mid;
      else lo = mid;
    }
    idx = lo;
  }
  if (idx < 0) idx = 0;
  if (idx > n - 1) idx = n - 1;
  if (order == 0) return cplx{poly[2 * idx], poly[2 * idx + 1]};
  const double f = t - tl[2 * idx];
  double re = 0.0, im = 0.0;
  for (int i = 0; i <= order; ++i) {
    re = re * f + poly[2 * (i * n + idx)];
    im = im * f + poly[2 * (i * n + idx) + 1];
  }
  return cplx{re, im};
}

// Evaluate one program at time t.  Programs are validated on the host (stack
// depth <= COEF_STACK); the interpreter additionally clamps the stack index so a
// malformed program cannot write outside its frame.
static __device__ __noinline__ cplx eval_coef(const int* code, const double* consts, double t) {
  cplx st[COEF_STACK];
  int sp = 0;
  for (int pc = 0; pc < 4096; ++pc) {
    int op = code[pc];
    if (op == OP_END) break;
    if (op == OP_CONST) {
      int k = code[++pc];
      if (sp < COEF_STACK) st[sp++] = cplx{consts[2 * k], consts[2 * k + 1]};
      continue;
    }
    if (op == OP_T) {
      if (sp < COEF_STACK) st[sp++] = cplx{t, 0.0};
      continue;
    }
    if (op == OP_INTERP) {
      int k = code[++pc];
      if (sp < COEF_STACK) st[sp++] = interp_eval(consts, k, t);
      continue;
    }
    if (sp < 1) return cplx{0.0, 0.0};
    cplx a = st[sp - 1];
    switch (op) {
      case OP_NEG: st[sp - 1] = cplx{-a.re, -a.im}; continue;
      case OP_COS: st[sp - 1] = c_cos(a); continue;
      case OP_SIN: st[sp - 1] = c_sin(a); continue;
      case OP_EXP: st[sp - 1] = c_exp(a); continue;
      case OP_LOG: st[sp - 1] = c_log(a); continue;
      case OP_SQRT: st[sp - 1] = c_sqrt(a); continue;
      case OP_CONJ: st[sp - 1] = cplx{a.re, -a.im}; continue;
      case OP_REAL: st[sp - 1] = cplx{a.re, 0.0}; continue;
      case OP_IMAG: st[sp - 1] = cplx{a.im, 0.0}; continue;
      case OP_ABS: st[sp - 1] = cplx{hypot(a.re, a.im), 0.0}; continue;
      case OP_COSH: st[sp - 1] = c_cosh(a); continue;
      case OP_SINH: st[sp - 1] = c_sinh(a); continue;
      case OP_TANH: st[sp - 1] = c_div(c_sinh(a), c_cosh(a)); continue;
      case OP_TAN: st[sp - 1] = c_div(c_sin(a), c_cos(a)); continue;
      case OP_ARCTAN:
        if (a.im == 0.0) {
          st[sp - 1] = cplx{atan(a.re), 0.0};
        } else {  // atan(z) = i/2 [log(1 - iz) - log(1 + iz)]
          cplx l1 = c_log(cplx{1.0 + a.im, -a.re});
          cplx l2 = c_log(cplx{1.0 - a.im, a.re});
          cplx d = csub(l1, l2);
          st[sp - 1] = cplx{-0.5 * d.im, 0.5 * d.re};
        }
        continue;
      default: break;
    }
    if (sp < 2) return cplx{0.0, 0.0};
    cplx b = st[sp - 1];
    a = st[sp - 2];
    cplx r;
    switch (op) {
      case OP_ADD: r = cadd(a, b); break;
      case OP_SUB: r = csub(a, b); break;
      case OP_MUL: r = cmul(a, b); break;
      case OP_DIV: r = c_div(a, b); break;
      case OP_POW:
        if (a.im == 0.0 && b.im == 0.0 && (a.re > 0.0 || b.re == floor(b.re))) {
          r = cplx{pow(a.re, b.re), 0.0};
        } else if (a.re == 0.0 && a.im == 0.0) {
          r = cplx{0.0, 0.0};
        } else {
          r = c_exp(cmul(b, c_log(a)));
        }
        break;
      default: return cplx{0.0, 0.0};
    }
    st[sp - 2] = r;
    --sp;
  }
  return sp > 0 ? st[sp - 1] : cplx{0.0, 0.0};
}

// Index into row_ptr of the start of (group g, row r) for either layout.
__device__ __forceinline__ int rp_index(const qg_csr_groups& A, int g, int r) {
  return A.layout == QG_LAYOUT_ROW_MAJOR ? r * A.n_groups + g
                                         : g * ((int)A.n_rows + 1) + r;
}

// Coefficient of group g at time t; a NULL program table means all ones.
__device__ __forceinline__ cplx group_coef(const qg_csr_groups& A, int g, double t) {
  if (A.coef_code == nullptr) return cplx{1.0, 0.0};
  return eval_coef(A.coef_code + A.coef_start[g], A.coef_consts, t);
}

// Float-float accumulation for the mixed form: hi + lo += (fh + fl) * k with the
// product error from one FMA (TwoProduct) and the addition error from Knuth's
// TwoSum (Ogita, Rump & Oishi, "Accurate sum and dot product", SIAM J. Sci.
// Comput. 26 (2005)).  The _rn intrinsics keep the compiler from contracting
// the product into the sum.  Vern7's stage weights are large and of both signs,
// so a plain FP32 sum of f_j k_j loses several bits of the stage input; this
// keeps it to the final rounding to FP32.
__device__ __forceinline__ void ff_acc(float& hi, float& lo, float fh, float fl, float k) {
  const float p = __fmul_rn(fh, k);
  float pe = fmaf(fh, k, -p);
  pe = fmaf(fl, k, pe);
  const float sum = __fadd_rn(hi, p);
  const float bp = __fsub_rn(sum, hi);
  const float e = __fadd_rn(__fsub_rn(hi, __fsub_rn(sum, bp)), __fsub_rn(p, bp));
  hi = sum;
  lo = __fadd_rn(lo, __fadd_rn(e, pe));
}

// dt * a as a float pair from dt = dh + dl and a = ah + al (tableau hi/lo):
// hi = fl(dh ah), lo = the product's rounding error plus the cross terms.
__device__ __forceinline__ void ff_factor(float dh, float dl, float ah, float al, float& fh,
                                          float& fl) {
  fh = __fmul_rn(dh, ah);
  float e = fmaf(dh, ah, -fh);
  e = fmaf(dh, al, e);
  fl = fmaf(dl, ah, e);
}

// fl32(bh + bl + ih + il): TwoSum of the high parts, the low parts added to its
// error, one final rounding.
__device__ __forceinline__ float ff_round4(float bh, float bl, float ih, float il) {
  const float sum = __fadd_rn(bh, ih);
  const float bp = __fsub_rn(sum, bh);
  float e = __fadd_rn(__fsub_rn(bh, __fsub_rn(sum, bp)), __fsub_rn(ih, bp));
  e = __fadd_rn(e, __fadd_rn(bl, il));
  return __fadd_rn(sum, e);
}

__device__ __forceinline__ void split_f(double v, float& h, float& l) {
  h = (float)v;
  l = (float)(v - (double)h);
}

}  // namespace qg
