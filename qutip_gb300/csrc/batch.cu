// Batched, persistent adaptive Vern7: many independent small solves in one
// launch.  Each CTA owns a workspace slot and takes items (a system solved from
// an initial state, or one Monte-Carlo trajectory) from an atomic queue; every
// item runs the reference's integrator control flow with its own step size:
//   Explicit_RungeKutta.set_initial_value / _estimate_first_step / integrate /
//   _step_in_err / _compute_step / _prep_dense_out / _interpolate_step /
//   _recompute_safe_step   (qutip/solver/integrator/explicit_rk.pyx:204-467)
// and, for trajectories, MCIntegrator.integrate / _find_collapse_time /
// _do_collapse (qutip/solver/mcsolve.py:245-406) with numpy's PCG64 draws in the
// reference's order.
//
// Inside a CTA: one thread per state row for the generator matvec, whose
// epilogue forms the next stage input (fused as in the single-system kernel);
// FP64 block reductions for the error norm, state norms and expectation values;
// thread 0 runs the scalar step control in FP64 and publishes every decision in
// shared memory, so all threads follow one control path.  Every loop is bounded:
// steps per output (nsteps), bisection tries (norm_steps), jumps (max_jumps), a
// host-visible cancel flag checked at each output time.
#include <mutex>

#include "capi_internal.h"
#include "common.cuh"

namespace qg {

// --------------------------------------------------------------- PCG64 ------
// Published PCG XSL-RR 128/64 generator: s <- s*M + inc (mod 2^128) before each
// output; output rotr64(hi(s) ^ lo(s), s >> 122); random() = (x >> 11) * 2^-53.
struct Pcg {
  unsigned long long hi, lo, ihi, ilo;
};
__device__ inline unsigned long long pcg_next(Pcg& r) {
  const unsigned long long MH = 0x2360ED051FC65DA4ULL, ML = 0x4385DF649FCCF645ULL;
  const unsigned long long lo = r.lo * ML;
  unsigned long long hi = __umul64hi(r.lo, ML) + r.lo * MH + r.hi * ML;
  const unsigned long long nlo = lo + r.ilo;
  hi += r.ihi + (nlo < lo ? 1ULL : 0ULL);
  r.lo = nlo;
  r.hi = hi;
  const unsigned long long x = hi ^ nlo;
  const unsigned rot = (unsigned)(hi >> 58);
  return (x >> rot) | (x << ((64u - rot) & 63u));
}
__device__ inline double pcg_random(Pcg& r) {
  return (double)(pcg_next(r) >> 11) * (1.0 / 9007199254740992.0);
}

// ------------------------------------------------------------ workspace -----
__host__ __device__ inline int64_t align256(int64_t b) { return (b + 255) & ~(int64_t)255; }

struct SlotLayout {
  int64_t y, ys, k, ytmp, ctmp, total;
};
__host__ __device__ inline SlotLayout slot_layout(int64_t n, int dt) {
  const int64_t es = dt == QG_C128 ? 16 : 8;
  SlotLayout L;
  L.y = 0;                                  // 2 state buffers (complex128)
  L.ys = L.y + align256(2 * n * 16);        // 2 stage-dtype shadows (mixed form)
  L.k = L.ys + align256(2 * n * es);        // 16 stage derivatives
  L.ytmp = L.k + align256(16 * n * es);     // 2 stage inputs
  L.ctmp = L.ytmp + align256(2 * n * es);   // 2 complex128 temporaries (MC)
  L.total = L.ctmp + align256(2 * n * 16);
  return L;
}

// ------------------------------------------------------------- control ------
struct Ctl {
  double t, t_prev, t_front, dt_safe, dt_int, err, red;
  double fa[16], fe[16];   // stage factors (FP64); float copies below
  float faf[16], fef[16];
  double bf[16];           // dense-output factors of the current output
  int status, cur, interp_ready, out_front, nsteps_done, rhs, steps_total;
  int flag;                // generic decision broadcast
};

template <int DT, int BB>
struct Ctx {
  using ST = typename elem<DT>::T;
  using CT = typename elem<DT>::R;
  static constexpr bool MIXED = (DT == QG_C64);
  const qg_batch* B;
  const qg_batch_system* S;
  int n, d, G;
  double2* y[2];
  ST* ys[2];
  ST* k;
  ST* ytmp;
  double2* ctmp[2];
  Ctl* c;
  double* red;           // [BB/32]
  double2* coef;         // [QG_MAX_GROUPS] FP64 coefficient values (stage time)
  const ST* opval;
};

template <int BB>
__device__ __forceinline__ double bsum(double v, double* red) {
  return block_sum<BB>(v, red);  // result valid in thread 0
}

// coefficients of the system's groups at time t -> shared memory
template <int DT, int BB>
__device__ void load_coef(Ctx<DT, BB>& X, double t) {
  if (threadIdx.x < X.G) {
    cplx c{1.0, 0.0};
    if (X.S->coef_off >= 0) {
      const int st = __ldg(X.B->coef_start + X.S->coef_off + threadIdx.x);
      c = eval_coef(X.B->coef_code + st, X.B->coef_consts, t);
    }
    X.coef[threadIdx.x] = make_double2(c.re, c.im);
  }
  __syncthreads();
}

// row r of A(t) x (coefficients already loaded), in the compute type CT
template <int DT, int BB, typename XT>
__device__ __forceinline__ void row_matvec(const Ctx<DT, BB>& X, int r, const XT* x,
                                           typename elem<DT>::R& ar, typename elem<DT>::R& ai) {
  using CT = typename elem<DT>::R;
  ar = 0;
  ai = 0;
  const int* rp = X.B->op_rp + X.S->rp_off + (int64_t)r * X.G;
  for (int g = 0; g < X.G; ++g) {
    const int s = __ldg(rp + g), e = __ldg(rp + g + 1);
    CT gr = 0, gi = 0;
    for (int p = s; p < e; ++p) {
      const auto v = __ldg(X.opval + p);
      const auto xv = x[__ldg(X.B->op_col + p)];
      gr = fma((CT)v.x, (CT)xv.x, gr);
      gr = fma(-(CT)v.y, (CT)xv.y, gr);
      gi = fma((CT)v.x, (CT)xv.y, gi);
      gi = fma((CT)v.y, (CT)xv.x, gi);
    }
    const CT cr = (CT)X.coef[g].x, ci = (CT)X.coef[g].y;
    ar += cr * gr - ci * gi;
    ai += cr * gi + ci * gr;
  }
}

template <typename T>
__device__ __forceinline__ void st2(T* p, double re, double im);
template <>
__device__ __forceinline__ void st2<double2>(double2* p, double re, double im) {
  *p = make_double2(re, im);
}
template <>
__device__ __forceinline__ void st2<float2>(float2* p, double re, double im) {
  *p = make_float2((float)re, (float)im);
}

// k_j = A(t) x for an arbitrary stage-dtype input (first-step estimate)
template <int DT, int BB>
__device__ void matvec_to_k(Ctx<DT, BB>& X, double t, const typename elem<DT>::T* x, int j) {
  using CT = typename elem<DT>::R;
  load_coef(X, t);
  for (int r = threadIdx.x; r < X.n; r += BB) {
    CT ar, ai;
    row_matvec(X, r, x, ar, ai);
    st2(X.k + (int64_t)j * X.n + r, (double)ar, (double)ai);
  }
  __syncthreads();
}

// stage factors -> shared memory (thread 0)
template <int DT, int BB>
__device__ void set_factors(Ctx<DT, BB>& X, int stage, double dt) {
  if (threadIdx.x < 16) {
    const int j = threadIdx.x;
    double a = 0.0, e = 0.0;
    if (stage == RK_STEP - 1) {
      if (j < RK_STEP) {
        a = dt * VERN7_B[j];
        e = dt * VERN7_E[j];
      }
    } else if (stage + 1 < RK_EXTRA_STEP && j <= stage) {
      a = dt * VERN7_A[stage + 1][j];
    }
    X.c->fa[j] = a;
    X.c->fe[j] = e;
    X.c->faf[j] = (float)a;
    X.c->fef[j] = (float)e;
  }
  __syncthreads();
}

template <int DT, int BB>
__device__ __forceinline__ typename elem<DT>::R factor_a(const Ctx<DT, BB>& X, int j) {
  if constexpr (DT == QG_C64) return X.c->faf[j];
  else return X.c->fa[j];
}
template <int DT, int BB>
__device__ __forceinline__ typename elem<DT>::R factor_e(const Ctx<DT, BB>& X, int j) {
  if constexpr (DT == QG_C64) return X.c->fef[j];
  else return X.c->fe[j];
}

// One fused stage: k_s = A(t_prev + c_s dt) x_s and the next stage input, or at
// s == 9 y_front and the WRMS error (-> X.c->err).
template <int DT, int BB>
__device__ __noinline__ void stage(Ctx<DT, BB>& X, int s, double dt) {
  using ST = typename elem<DT>::T;
  using CT = typename elem<DT>::R;
  constexpr bool MIXED = Ctx<DT, BB>::MIXED;
  const int cur = X.c->cur;
  set_factors(X, s, dt);
  load_coef(X, X.c->t_prev + VERN7_C[s] * dt);
  const ST* x;
  if (s == 0) {
    if constexpr (MIXED) x = X.ys[cur];
    else x = reinterpret_cast<const ST*>(X.y[cur]);
  } else {
    x = X.ytmp + (int64_t)(s & 1) * X.n;
  }
  ST* out = X.ytmp + (int64_t)((s + 1) & 1) * X.n;
  const int64_t n = X.n;
  double err_acc = 0.0;
  for (int r = threadIdx.x; r < X.n; r += BB) {
    CT ar, ai;
    row_matvec(X, r, x, ar, ai);
    st2(X.k + s * n + r, (double)ar, (double)ai);
    const ST ks = X.k[s * n + r];
    if (s != RK_STEP - 1 && s != RK_EXTRA_STEP - 1) {
      CT vr, vi;
      if constexpr (MIXED) {
        vr = X.ys[cur][r].x;
        vi = X.ys[cur][r].y;
      } else {
        vr = (CT)X.y[cur][r].x;
        vi = (CT)X.y[cur][r].y;
      }
      for (int j = 0; j <= s; ++j) {
        const CT f = factor_a(X, j);
        if (f != (CT)0) {
          const ST kj = (j == s) ? ks : X.k[j * n + r];
          vr = fma(f, (CT)kj.x, vr);
          vi = fma(f, (CT)kj.y, vi);
        }
      }
      st2(out + r, (double)vr, (double)vi);
    } else if (s == RK_STEP - 1) {
      CT ir = 0, ii = 0, er = 0, ei = 0;
      double yr, yi;
      if constexpr (MIXED) {
        for (int j = 0; j < RK_STEP; ++j) {
          const CT fb = factor_a(X, j), fq = factor_e(X, j);
          if (fb == (CT)0 && fq == (CT)0) continue;
          const ST kj = (j == s) ? ks : X.k[j * n + r];
          ir = fma(fb, (CT)kj.x, ir);
          ii = fma(fb, (CT)kj.y, ii);
          er = fma(fq, (CT)kj.x, er);
          ei = fma(fq, (CT)kj.y, ei);
        }
        yr = X.y[cur][r].x + (double)ir;
        yi = X.y[cur][r].y + (double)ii;
        X.ys[cur ^ 1][r] = make_float2((float)yr, (float)yi);
      } else {
        yr = X.y[cur][r].x;
        yi = X.y[cur][r].y;
        for (int j = 0; j < RK_STEP; ++j) {
          const double fb = X.c->fa[j], fq = X.c->fe[j];
          if (fb == 0.0 && fq == 0.0) continue;
          const ST kj = (j == s) ? ks : X.k[j * n + r];
          if (fb != 0.0) {
            yr = fma(fb, (double)kj.x, yr);
            yi = fma(fb, (double)kj.y, yi);
          }
          if (fq != 0.0) {
            er = fma((CT)fq, (CT)kj.x, er);
            ei = fma((CT)fq, (CT)kj.y, ei);
          }
        }
      }
      X.y[cur ^ 1][r] = make_double2(yr, yi);
      const double w = sqrt((double)er * er + (double)ei * ei) /
                       (X.S->atol + X.S->rtol * sqrt(yr * yr + yi * yi));
      err_acc += w * w;
    }
  }
  if (s == RK_STEP - 1) {
    const double tot = bsum<BB>(err_acc, X.red);
    if (threadIdx.x == 0) X.c->err = sqrt(tot / (double)X.n);
  }
  if (threadIdx.x == 0) X.c->rhs += 1;
  __syncthreads();
}

// out (complex128 or stage dtype) = base + sum_{j<nk} f_j k_j, with f in X.c->bf
template <int DT, int BB, typename OT, typename BT>
__device__ void combine(Ctx<DT, BB>& X, OT* out, const BT* base, int nk) {
  for (int r = threadIdx.x; r < X.n; r += BB) {
    double vr = (double)base[r].x, vi = (double)base[r].y;
    for (int j = 0; j < nk; ++j) {
      const double f = X.c->bf[j];
      if (f != 0.0) {
        vr = fma(f, (double)X.k[(int64_t)j * X.n + r].x, vr);
        vi = fma(f, (double)X.k[(int64_t)j * X.n + r].y, vi);
      }
    }
    st2(out + r, vr, vi);
  }
  __syncthreads();
}

// entry i of the current state: y_front, or y_prev + sum_j bf_j k_j
template <int DT, int BB>
__device__ __forceinline__ double2 state_at(const Ctx<DT, BB>& X, int i) {
  const int cur = X.c->cur;
  if (X.c->out_front) return X.y[cur ^ 1][i];
  double vr = X.y[cur][i].x, vi = X.y[cur][i].y;
  for (int j = 0; j < RK_EXTRA_STEP; ++j) {
    const double f = X.c->bf[j];
    if (f != 0.0) {
      vr = fma(f, (double)X.k[(int64_t)j * X.n + i].x, vr);
      vi = fma(f, (double)X.k[(int64_t)j * X.n + i].y, vi);
    }
  }
  return make_double2(vr, vi);
}

template <int DT, int BB>
__device__ double state_norm2(Ctx<DT, BB>& X) {
  double acc = 0.0;
  for (int r = threadIdx.x; r < X.n; r += BB) {
    const double2 v = state_at(X, r);
    acc += v.x * v.x + v.y * v.y;
  }
  const double tot = bsum<BB>(acc, X.red);
  if (threadIdx.x == 0) X.c->red = tot;
  __syncthreads();
  return X.c->red;
}

template <int BB>
__device__ double vec_norm2(const double2* v, int n, double* red, Ctl* c) {
  double acc = 0.0;
  for (int r = threadIdx.x; r < n; r += BB) acc += v[r].x * v[r].x + v[r].y * v[r].y;
  const double tot = bsum<BB>(acc, red);
  if (threadIdx.x == 0) c->red = tot;
  __syncthreads();
  return c->red;
}

// ||x||^2 of a stage-dtype vector
template <int DT, int BB>
__device__ double stage_norm2(Ctx<DT, BB>& X, const typename elem<DT>::T* v) {
  double acc = 0.0;
  for (int r = threadIdx.x; r < X.n; r += BB)
    acc += (double)v[r].x * (double)v[r].x + (double)v[r].y * (double)v[r].y;
  const double tot = bsum<BB>(acc, X.red);
  if (threadIdx.x == 0) X.c->red = tot;
  __syncthreads();
  return X.c->red;
}

// ------------------------------------------------------ integrator (RK) ------
// set_initial_value: state from src (complex128), first-step estimate
template <int DT, int BB>
__device__ __noinline__ void set_initial(Ctx<DT, BB>& X, const double2* src, double t) {
  using ST = typename elem<DT>::T;
  constexpr bool MIXED = Ctx<DT, BB>::MIXED;
  const int cur = X.c->cur;
  for (int r = threadIdx.x; r < X.n; r += BB) {
    const double2 v = src[r];
    X.y[cur][r] = v;
    X.y[cur ^ 1][r] = v;
    if constexpr (MIXED) {
      X.ys[cur][r] = make_float2((float)v.x, (float)v.y);
      X.ys[cur ^ 1][r] = make_float2((float)v.x, (float)v.y);
    }
  }
  if (threadIdx.x == 0) {
    X.c->t = X.c->t_prev = X.c->t_front = t;
    X.c->dt_int = 0.0;
    X.c->interp_ready = 0;
    X.c->out_front = 1;
    X.c->status = QG_NORMAL;
  }
  __syncthreads();
  // _estimate_first_step (explicit_rk.pyx:232-276)
  const double atol = X.S->atol, rtol = X.S->rtol;
  double norm = sqrt(vec_norm2<BB>(X.y[cur], X.n, X.red, X.c));
  const double tol = atol + norm * rtol;
  const ST* x0;
  if constexpr (MIXED) x0 = X.ys[cur];
  else x0 = reinterpret_cast<const ST*>(X.y[cur]);
  matvec_to_k(X, t, x0, 0);
  if (norm <= atol) norm = 1.0;
  double tmp = sqrt(stage_norm2(X, X.k));
  double fact = 1.0;
  for (int i = 1; i <= RK_ORDER; ++i) fact *= i;
  double dt1;
  if (tmp >= atol * 1e-6)
    dt1 = pow(tol * fact * pow(norm, (double)RK_ORDER), 1.0 / (RK_ORDER + 1)) / tmp;
  else
    dt1 = pow(tol * fact, 1.0 / (RK_ORDER + 1)) * norm * 0.5;
  const double t1 = t + dt1 / 100;
  if (threadIdx.x == 0) {
    for (int j = 0; j < 16; ++j) X.c->bf[j] = 0.0;
    X.c->bf[0] = dt1 / 100;
  }
  __syncthreads();
  ST* yt = X.ytmp + X.n;
  combine(X, yt, x0, 1);
  matvec_to_k(X, t1, yt, 1);
  tmp = sqrt(stage_norm2(X, X.k + X.n));
  double dt2;
  if (tmp >= atol * 1e-6)
    dt2 = pow(tol * fact * pow(norm, (double)RK_ORDER), 1.0 / (RK_ORDER + 1)) / tmp;
  else
    dt2 = dt1;
  double dt = fmin(dt1, dt2);
  dt = fmax(1e-15, dt);  // min_step defaults to 1e-15 (explicit_rk.pyx:133)
  if (threadIdx.x == 0) {
    X.c->dt_safe = dt;
    X.c->rhs += 2;
  }
  __syncthreads();
}

template <int DT, int BB>
__device__ __noinline__ void prep_dense_out(Ctx<DT, BB>& X) {
  using ST = typename elem<DT>::T;
  const double dt = X.c->dt_int;
  const int cur = X.c->cur;
  if (threadIdx.x < 16) X.c->bf[threadIdx.x] = threadIdx.x < RK_STEP ? dt * VERN7_A[RK_STEP][threadIdx.x] : 0.0;
  __syncthreads();
  const ST* base;
  if constexpr (Ctx<DT, BB>::MIXED) base = X.ys[cur];
  else base = reinterpret_cast<const ST*>(X.y[cur]);
  combine(X, X.ytmp + (int64_t)(RK_STEP & 1) * X.n, base, RK_STEP);
  for (int s = RK_STEP; s < RK_EXTRA_STEP; ++s) stage(X, s, dt);
  if (threadIdx.x == 0) X.c->interp_ready = 1;
  __syncthreads();
}

// dense-output factors at t (Horner in tau, explicit_rk.pyx:412-430)
template <int DT, int BB>
__device__ void set_interp(Ctx<DT, BB>& X, double t) {
  if (threadIdx.x < RK_EXTRA_STEP) {
    const int i = threadIdx.x;
    const double tau = (t - X.c->t_prev) / X.c->dt_int;
    double acc = 0.0;
    for (int j = DENSE_ORDER - 1; j >= 0; --j) {
      acc += VERN7_BI[i][j];
      acc *= tau;
    }
    X.c->bf[i] = X.c->dt_int * acc;
  }
  if (threadIdx.x == 0) {
    X.c->out_front = 0;
    X.c->t = t;
  }
  __syncthreads();
}

// _step_in_err (explicit_rk.pyx:333-356) with interpolate=True time steps
template <int DT, int BB>
__device__ void step_in_err(Ctx<DT, BB>& X, int& nsteps_left) {
  int nsteps = 0;
  while (true) {
    const double dt = X.c->dt_safe;
    for (int s = 0; s < RK_STEP; ++s) stage(X, s, dt);
    if (threadIdx.x == 0) {
      Ctl* c = X.c;
      c->t_front = c->t_prev + dt;
      const double err = c->err;
      c->dt_int = dt;
      double factor;
      if (err == 0.0) factor = 10.0;
      else factor = fmax(0.2, fmin(10.0, 0.9 * pow(err, -1.0 / (RK_ORDER + 1))));
      c->dt_safe = fmax(1e-15, dt * factor);
      c->nsteps_done += 1;
      c->steps_total += 1;
      c->flag = 0;  // 0: retry, 1: accepted, 2: failed
      if (dt == 1e-15 && err > 1.0) {
        c->status = QG_DT_UNDERFLOW;
        c->flag = 2;
      } else if (++nsteps > nsteps_left) {
        c->status = QG_TOO_MUCH_WORK;
        c->flag = 2;
      } else if (err < 1.0) {
        c->flag = 1;
      }
      c->interp_ready = 0;
    }
    __syncthreads();
    if (X.c->flag != 0) break;
  }
  // the same count on every thread, read after the loop's final barrier
  nsteps_left -= X.c->nsteps_done;  // caller resets nsteps_done per integrate call
}

// integrate (explicit_rk.pyx:278-331); on return the state at X.c->t is
// y_front (out_front) or the dense output with factors bf.
template <int DT, int BB>
__device__ void integrate(Ctx<DT, BB>& X, double t, bool step) {
  if (t == X.c->t) return;
  if (t < X.c->t_prev) {
    if (threadIdx.x == 0) X.c->status = QG_OUTSIDE_RANGE;
    __syncthreads();
    return;
  }
  if (t < X.c->t_front) {
    if (!X.c->interp_ready) prep_dense_out(X);
    set_interp(X, t);
    return;
  }
  if (threadIdx.x == 0) X.c->status = QG_NORMAL;
  __syncthreads();
  if (step && X.c->t < X.c->t_front && t > X.c->t_front) t = X.c->t_front;
  int nsteps_left = X.S->nsteps;
  while (X.c->t_front < t && X.c->status >= 0) {
    if (threadIdx.x == 0) {
      X.c->cur ^= 1;  // y_prev <- y_front (buffer swap)
      X.c->t_prev = X.c->t_front;
      X.c->nsteps_done = 0;
    }
    __syncthreads();
    step_in_err(X, nsteps_left);
    if (step) break;
  }
  if (X.c->status < 0) return;
  if (X.c->t_front > t) {
    prep_dense_out(X);
    set_interp(X, t);
  } else {
    if (threadIdx.x == 0) {
      X.c->out_front = 1;
      X.c->t = X.c->t_front;
    }
    __syncthreads();
  }
}

// ------------------------------------------------------------- outputs ------
// expectation values of the current state into out[o] (raw; host normalises)
template <int DT, int BB>
__device__ __noinline__ void record(Ctx<DT, BB>& X, double2* out, bool ket) {
  const int ne = X.S->n_eops;
  const int d = X.d;
  for (int e = 0; e < ne; ++e) {
    const int* rp = X.B->eop_rp + X.S->eop_rp_off + (int64_t)e * (d + 1);
    double ar = 0.0, ai = 0.0;
    for (int r = threadIdx.x; r < d; r += BB) {
      const int s = __ldg(rp + r), en = __ldg(rp + r + 1);
      double sr = 0.0, si = 0.0;
      for (int p = s; p < en; ++p) {
        const int c = __ldg(X.B->eop_col + p);
        const double vr = __ldg(X.B->eop_val + 2 * p), vi = __ldg(X.B->eop_val + 2 * p + 1);
        const double2 z = state_at(X, ket ? c : c + r * d);
        sr += vr * z.x - vi * z.y;
        si += vr * z.y + vi * z.x;
      }
      if (ket) {
        const double2 pr = state_at(X, r);
        const double tr = pr.x * sr + pr.y * si, ti = pr.x * si - pr.y * sr;
        sr = tr;
        si = ti;
      }
      ar += sr;
      ai += si;
    }
    const double tr_ = bsum<BB>(ar, X.red);
    const double ti_ = bsum<BB>(ai, X.red);
    if (threadIdx.x == 0) out[e] = make_double2(tr_, ti_);
  }
  double ar = 0.0, ai = 0.0;
  if (ket) {
    for (int r = threadIdx.x; r < X.n; r += BB) {
      const double2 z = state_at(X, r);
      ar += z.x * z.x + z.y * z.y;
    }
  } else {
    for (int r = threadIdx.x; r < d; r += BB) {
      const double2 z = state_at(X, r + r * d);
      ar += z.x;
      ai += z.y;
    }
  }
  const double tr_ = bsum<BB>(ar, X.red);
  const double ti_ = bsum<BB>(ai, X.red);
  if (threadIdx.x == 0) out[ne] = make_double2(tr_, ti_);
  __syncthreads();
}

// ------------------------------------------------------------------ MC -------
// ||c_i psi||^2 for psi in ctmp[0]; optionally store c_i psi in ctmp[1]
template <int DT, int BB>
__device__ double cop_apply(Ctx<DT, BB>& X, int i, bool store) {
  const int d = X.d;
  const int* rp = X.B->cop_rp + X.S->cop_rp_off + (int64_t)i * (d + 1);
  double acc = 0.0;
  for (int r = threadIdx.x; r < d; r += BB) {
    const int s = __ldg(rp + r), e = __ldg(rp + r + 1);
    double sr = 0.0, si = 0.0;
    for (int p = s; p < e; ++p) {
      const int c = __ldg(X.B->cop_col + p);
      const double vr = __ldg(X.B->cop_val + 2 * p), vi = __ldg(X.B->cop_val + 2 * p + 1);
      const double2 z = X.ctmp[0][c];
      sr += vr * z.x - vi * z.y;
      si += vr * z.y + vi * z.x;
    }
    if (store) X.ctmp[1][r] = make_double2(sr, si);
    acc += sr * sr + si * si;
  }
  const double tot = bsum<BB>(acc, X.red);
  if (threadIdx.x == 0) X.c->red = tot;
  __syncthreads();
  return X.c->red;
}

}  // namespace qg

using namespace qg;

namespace qg {

template <int DT, int BB>
__global__ void __launch_bounds__(BB) batch_vern7_kernel(qg_batch B) {
  using ST = typename elem<DT>::T;
  __shared__ Ctl ctl;
  __shared__ double red[BB / 32];
  __shared__ double2 coef[QG_MAX_GROUPS];
  __shared__ int item_s;
  __shared__ Pcg rng;
  __shared__ double target;

  const SlotLayout L = slot_layout(B.max_n, DT);
  char* slot = static_cast<char*>(B.work) + (int64_t)blockIdx.x * L.total;
  Ctx<DT, BB> X;
  X.B = &B;
  X.c = &ctl;
  X.red = red;
  X.coef = coef;
  X.opval = static_cast<const ST*>(B.op_val);
  X.y[0] = reinterpret_cast<double2*>(slot + L.y);
  X.y[1] = X.y[0] + B.max_n;
  X.ys[0] = reinterpret_cast<ST*>(slot + L.ys);
  X.ys[1] = X.ys[0] + B.max_n;
  X.k = reinterpret_cast<ST*>(slot + L.k);
  X.ytmp = reinterpret_cast<ST*>(slot + L.ytmp);
  X.ctmp[0] = reinterpret_cast<double2*>(slot + L.ctmp);
  X.ctmp[1] = X.ctmp[0] + B.max_n;

  while (true) {
    if (threadIdx.x == 0) {
      int it = (int)atomicAdd(B.queue, 1u);
      if (B.cancel && *B.cancel) it = B.n_items;  // stop taking work
      item_s = it;
    }
    __syncthreads();
    const int item = item_s;
    if (item >= B.n_items) break;
    const qg_batch_item I = B.items[item];
    const qg_batch_system* S = B.systems + I.system;
    X.S = S;
    X.n = S->n;
    X.d = S->d;
    X.G = S->n_groups;
    const bool ket = S->kind == 1;
    double2* out = reinterpret_cast<double2*>(B.out + 2 * I.out_off);
    const double* tl = B.tlist + S->tlist_off;
    const int ne1 = S->n_eops + 1;
    int njumps = 0;
    if (threadIdx.x == 0) {
      ctl.cur = 0;
      ctl.rhs = 0;
      ctl.nsteps_done = 0;
      ctl.steps_total = 0;
      rng = Pcg{I.rng_state_hi, I.rng_state_lo, I.rng_inc_hi, I.rng_inc_lo};
      target = ket ? pcg_random(rng) : 0.0;  // MCIntegrator.set_state draws first
    }
    __syncthreads();
    set_initial(X, reinterpret_cast<const double2*>(B.y0) + I.y0_off, tl[0]);
    record(X, out, ket);
    for (int o = 1; o < S->n_out && ctl.status >= 0; ++o) {
      const double t = tl[o];
      if (B.cancel) {  // host-visible cancel flag, read once per output by thread 0
        if (threadIdx.x == 0 && *B.cancel) ctl.status = QG_TIMEOUT;
        __syncthreads();
        if (ctl.status < 0) break;
      }
      if (!ket) {
        integrate(X, t, false);
      } else {
        // MCIntegrator.integrate (mcsolve.py:286-302)
        double t_old = ctl.t;
        double norm_old = state_norm2(X);
        while (t_old < t && ctl.status >= 0) {
          integrate(X, t, true);
          if (ctl.status < 0) break;
          const double t_step = ctl.t;
          const double nrm = state_norm2(X);
          if (nrm <= target) {
            // _find_collapse_time (mcsolve.py:321-369)
            double tp = t_old, tf = t_step, no = norm_old, nn = nrm, t_guess = tf;
            int tries = 0;
            while (tries < B.norm_steps) {
              ++tries;
              if ((tf - tp) < B.norm_t_tol) {
                t_guess = tf;
                break;
              }
              const double dtb = tf - tp;
              double ratio = log(no / target) / log(no / nn);
              if (ratio < B.norm_min_step) ratio = B.norm_min_step;
              if (ratio > 1.0 - B.norm_min_step) ratio = 1.0 - B.norm_min_step;
              t_guess = tp + dtb * ratio;
              if ((t_guess - tp) < B.norm_t_tol) t_guess = tp + B.norm_t_tol;
              integrate(X, t_guess, true);
              if (ctl.status < 0) break;
              const double n2 = state_norm2(X);
              if (fabs(target - n2) < B.norm_tol * target) break;
              if (n2 < target) {
                tf = t_guess;
                nn = n2;
              } else {
                tp = t_guess;
                no = n2;
              }
            }
            if (ctl.status < 0) break;
            if (tries >= B.norm_steps) {
              if (threadIdx.x == 0) ctl.status = QG_NORM_SEARCH_FAILED;
              __syncthreads();
              break;
            }
            // _do_collapse (mcsolve.py:371-406): psi = state at t_guess
            for (int r = threadIdx.x; r < X.n; r += BB) X.ctmp[0][r] = state_at(X, r);
            __syncthreads();
            int which = 0;
            if (S->n_cops > 1) {
              double probs[16];
              double sum = 0.0;
              const int nc = S->n_cops < 16 ? S->n_cops : 16;
              for (int i = 0; i < nc; ++i) {
                probs[i] = cop_apply(X, i, false);
                sum += probs[i];
              }
              if (threadIdx.x == 0) {
                double tgt = sum * pcg_random(rng) - probs[0];
                int w = 0;
                while (tgt > 0 && w < nc - 1) {
                  ++w;
                  tgt -= probs[w];
                }
                ctl.flag = w;
              }
              __syncthreads();
              which = ctl.flag;
            }
            const double new_n2 = cop_apply(X, which, true);
            const double new_norm = sqrt(new_n2);
            const double2* src;
            if (new_norm < B.mc_corr_eps) {
              const double pn = sqrt(vec_norm2<BB>(X.ctmp[0], X.n, X.red, X.c));
              for (int r = threadIdx.x; r < X.n; r += BB)
                X.ctmp[1][r] = make_double2(X.ctmp[0][r].x / pn, X.ctmp[0][r].y / pn);
            } else {
              for (int r = threadIdx.x; r < X.n; r += BB)
                X.ctmp[1][r] = make_double2(X.ctmp[1][r].x / new_norm, X.ctmp[1][r].y / new_norm);
              if (threadIdx.x == 0) {
                if (njumps < B.max_jumps) {
                  B.jump_t[(int64_t)item * B.max_jumps + njumps] = t_guess;
                  B.jump_which[(int64_t)item * B.max_jumps + njumps] = which;
                } else {
                  ctl.status = QG_JUMP_OVERFLOW;
                }
                target = pcg_random(rng);
              }
              ++njumps;
            }
            __syncthreads();
            src = X.ctmp[1];
            set_initial(X, src, t_guess);
            if (ctl.status < 0) break;
            t_old = ctl.t;
            norm_old = 1.0;
          } else {
            t_old = t_step;
            norm_old = nrm;
          }
        }
      }
      if (ctl.status < 0) break;
      record(X, out + (int64_t)o * ne1, ket);
    }
    if (threadIdx.x == 0) {
      int32_t* st = B.status + 4 * (int64_t)item;
      st[0] = ctl.status < 0 ? ctl.status : 0;
      st[1] = ctl.steps_total;
      st[2] = ctl.rhs;
      st[3] = njumps;
    }
    __syncthreads();
  }
  // the last CTA to finish resets the queue words for the next launch
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(B.queue + 1, 1u) == gridDim.x - 1) {
      B.queue[0] = 0u;
      B.queue[1] = 0u;
    }
  }
}

}  // namespace qg

// ------------------------------------------------- allocation-free variant --
// Workspace and queue words of qg_batch_vern7_noalloc.  Loading the library
// reserves these on every GPU it is used on, until the process exits.
namespace qg {
constexpr size_t NOALLOC_WORK_BYTES = (size_t)QG_NOALLOC_WORK_BYTES;
static __device__ __align__(256) unsigned char g_noalloc_work[NOALLOC_WORK_BYTES];
static __device__ __align__(256) unsigned int g_noalloc_queue[4];

// Device addresses of the arrays above, looked up once per device with that
// device current (the host-side names are stand-ins, not device addresses).
struct NoallocAddr {
  void* work = nullptr;
  unsigned int* queue = nullptr;
};
static NoallocAddr g_noalloc_addr[64];
static std::mutex g_noalloc_mu;

static int noalloc_setup(int dev, NoallocAddr& out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  NoallocAddr& a = g_noalloc_addr[dev];
  if (!a.work) {
    void* w = nullptr;
    void* q = nullptr;
    if (cudaGetSymbolAddress(&w, g_noalloc_work) != cudaSuccess || !w)
      return set_error(QG_ERR_CUDA, "cudaGetSymbolAddress failed for the static workspace");
    if (cudaGetSymbolAddress(&q, g_noalloc_queue) != cudaSuccess || !q)
      return set_error(QG_ERR_CUDA, "cudaGetSymbolAddress failed for the static queue words");
    a.work = w;
    a.queue = static_cast<unsigned int*>(q);
  }
  out = a;
  return QG_OK;
}
}  // namespace qg

extern "C" int qg_batch_vern7_noalloc(const qg_batch* B, void* stream) {
  if (!B || !B->systems || !B->items || !B->op_rp || !B->op_col || !B->op_val || !B->tlist ||
      !B->y0 || !B->out || !B->status)
    return set_error(QG_ERR_ARG, "null batch pointer");
  if (B->dtype != QG_C128 && B->dtype != QG_C64)
    return set_error(QG_ERR_UNSUPPORTED, "batch dtype must be QG_C128 or QG_C64");
  if (B->n_items < 0 || B->max_n <= 0) return set_error(QG_ERR_ARG, "bad batch sizes");
  if (B->max_jumps > 0 && (!B->jump_t || !B->jump_which))
    return set_error(QG_ERR_ARG, "jump record buffers missing");
  const int64_t slot = slot_layout(B->max_n, B->dtype).total;
  if (slot > (int64_t)NOALLOC_WORK_BYTES)
    return set_error(QG_ERR_ARG,
                     "max_n too large: one workspace slot exceeds the static workspace "
                     "(QG_NOALLOC_WORK_BYTES); use qg_batch_vern7 with caller-owned memory");
  if (B->n_items == 0) return QG_OK;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
    return set_error(QG_ERR_CUDA, "no current CUDA device");
  NoallocAddr a;
  int rc = noalloc_setup(dev, a);
  if (rc) return rc;
  int occ = qg_batch_max_slots(B->max_n, B->dtype);
  if (occ <= 0) return occ < 0 ? occ : set_error(QG_ERR_CUDA, "no resident CTA");
  int64_t slots = (int64_t)NOALLOC_WORK_BYTES / slot;
  if (slots > occ) slots = occ;
  if (slots > B->n_items) slots = B->n_items;
  qg_batch b = *B;
  b.work = a.work;
  b.queue = a.queue;
  b.n_slots = (int32_t)slots;
  cudaStream_t st = (cudaStream_t)stream;
  // the queue words must start at zero (a previous launch leaves them zero; clear anyway)
  if (cudaMemsetAsync(a.queue, 0, 4 * sizeof(unsigned int), st) != cudaSuccess)
    return set_error(QG_ERR_CUDA, "clearing the static queue words failed");
  return qg_batch_vern7(&b, stream);
}

extern "C" int64_t qg_batch_slot_bytes(int64_t max_n, int dtype) {
  return slot_layout(max_n, dtype).total;
}

extern "C" int qg_batch_max_slots(int64_t max_n, int dtype) {
  int per_sm = 0;
  cudaError_t e;
  if (dtype == QG_C64)
    e = max_n <= 128 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                           &per_sm, batch_vern7_kernel<QG_C64, 128>, 128, 0)
                     : cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                           &per_sm, batch_vern7_kernel<QG_C64, 256>, 256, 0);
  else
    e = max_n <= 128 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                           &per_sm, batch_vern7_kernel<QG_C128, 128>, 128, 0)
                     : cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                           &per_sm, batch_vern7_kernel<QG_C128, 256>, 256, 0);
  if (e != cudaSuccess || per_sm <= 0) return set_error(QG_ERR_CUDA, "occupancy query failed");
  return sm_count() * per_sm;
}

extern "C" int qg_batch_vern7(const qg_batch* B, void* stream) {
  if (!B || !B->systems || !B->items || !B->op_rp || !B->op_col || !B->op_val || !B->tlist ||
      !B->y0 || !B->out || !B->status || !B->work || !B->queue)
    return set_error(QG_ERR_ARG, "null batch pointer");
  if (B->dtype != QG_C128 && B->dtype != QG_C64)
    return set_error(QG_ERR_UNSUPPORTED, "batch dtype must be QG_C128 or QG_C64");
  if (B->n_items < 0 || B->n_slots <= 0 || B->max_n <= 0)
    return set_error(QG_ERR_ARG, "bad batch sizes");
  if (B->max_jumps > 0 && (!B->jump_t || !B->jump_which))
    return set_error(QG_ERR_ARG, "jump record buffers missing");
  if (B->n_items == 0) return QG_OK;
  cudaStream_t st = (cudaStream_t)stream;
  const int bb = B->max_n <= 128 ? 128 : 256;
  if (B->dtype == QG_C64) {
    if (bb == 128) batch_vern7_kernel<QG_C64, 128><<<B->n_slots, 128, 0, st>>>(*B);
    else batch_vern7_kernel<QG_C64, 256><<<B->n_slots, 256, 0, st>>>(*B);
  } else {
    if (bb == 128) batch_vern7_kernel<QG_C128, 128><<<B->n_slots, 128, 0, st>>>(*B);
    else batch_vern7_kernel<QG_C128, 256><<<B->n_slots, 256, 0, st>>>(*B);
  }
  return check_launch("batch_vern7_kernel");
}
