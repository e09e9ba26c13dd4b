// Stochastic Schrodinger and master equations with the reference's explicit Platen scheme
// (qutip/solver/sode/_sode.pyx:58-120, Breuer & Petruccione eq. 7.47), drift and diffusion
// of qutip/solver/sode/ssystem.pyx:119-250.  A group of threads integrates one trajectory
// through n_steps fixed steps with the Wiener increments the host drew (the reference's own
// generator stream), so a launch covers a whole output interval of one or many
// trajectories.  A state of up to 64 entries is integrated by one warp (4 trajectories
// per CTA; syncs are __syncwarp), a larger one by a CTA of 256 threads.  Every vector
// operation follows the reference's order of operations
// (`_data.add(a, b, s)` is a + s b element by element, the complex scalars formed the way
// the reference forms them); CSR rows are summed in column order.
#include "capi_internal.h"
#include "common.cuh"

namespace qg {

constexpr int SDE_BLOCK = 256;   // CTA shape: one trajectory per CTA
constexpr int SDE_WARPS = 4;     // warp shape: one trajectory per warp, 4 per CTA
constexpr int SDE_WARP_MAX_N = 64;  // states up to this length take the warp shape

// A group of GS threads integrating one trajectory: a warp (GS = 32, syncs are
// __syncwarp, sums are XOR butterflies) or a CTA (GS = SDE_BLOCK).  Sums come back to
// every thread with the same bits.
template <int GS>
struct SdeGroup;
template <>
struct SdeGroup<32> {
  int rank;
  __device__ __forceinline__ void sync() const { __syncwarp(); }
  __device__ __forceinline__ double2 sum(double2 v, double*) const {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
      v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
    }
    return v;
  }
};
template <>
struct SdeGroup<SDE_BLOCK> {
  int rank;
  __device__ __forceinline__ void sync() const { __syncthreads(); }
  __device__ double2 sum(double2 v, double* red) const {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      v.x += __shfl_down_sync(0xffffffffu, v.x, o);
      v.y += __shfl_down_sync(0xffffffffu, v.y, o);
    }
    constexpr int W = SDE_BLOCK / 32;
    __syncthreads();  // earlier readers of red are done
    if ((threadIdx.x & 31) == 0) {
      red[threadIdx.x >> 5] = v.x;
      red[W + (threadIdx.x >> 5)] = v.y;
    }
    __syncthreads();
    double re = 0.0, im = 0.0;
    for (int w = 0; w < W; ++w) {
      re += red[w];
      im += red[W + w];
    }
    return make_double2(re, im);
  }
};

struct Sde {
  const qg_sde* S;
  int n, m;
  double2* F;   // drift output
  double2* D1;  // state + dt drift
  double2* VT;  // Platen support vector
  double2* TMP;
  double2* D2;  // m diffusion vectors
  double2* VP;  // m support vectors (+)
  double2* VM;  // m support vectors (-)
  double2* D2P; // m diffusions at VP_i
  double2* D2M; // m diffusions at VM_i
  double* red;  // reduction scratch (CTA shape)
};

__device__ __forceinline__ double2 cmul2(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// a + s b
__device__ __forceinline__ double2 axpy(double2 a, double2 s, double2 b) {
  const double2 t = cmul2(s, b);
  return make_double2(a.x + t.x, a.y + t.y);
}
__device__ __forceinline__ double2 axpy(double2 a, double s, double2 b) {
  return make_double2(a.x + s * b.x, a.y + s * b.y);
}

// y = rows [row0, row0 + n) of a CSR operator times x (x complete on entry)
template <int GS>
__device__ void csr_mv(const SdeGroup<GS>& g, const int* __restrict__ rp,
                       const int* __restrict__ col, const double2* __restrict__ val,
                       int64_t row0, const double2* x, double2* y, int n) {
  for (int r = g.rank; r < n; r += GS) {
    const int s = __ldg(rp + row0 + r), e = __ldg(rp + row0 + r + 1);
    double ar = 0.0, ai = 0.0;
    for (int p = s; p < e; ++p) {
      const double2 v = __ldg(val + p);
      const double2 z = x[__ldg(col + p)];
      ar += v.x * z.x - v.y * z.y;
      ai += v.x * z.y + v.y * z.x;
    }
    y[r] = make_double2(ar, ai);
  }
}

// SSE: <x| M_i |x> (M_i x goes through TMP)
template <int GS>
__device__ double2 expect_m(const SdeGroup<GS>& g, const Sde& q, int i, const double2* x) {
  const qg_sde& S = *q.S;
  g.sync();
  csr_mv(g, S.m_rp, S.m_col, static_cast<const double2*>(S.m_val), (int64_t)i * q.n, x, q.TMP,
         q.n);
  double2 acc = make_double2(0.0, 0.0);
  for (int r = g.rank; r < q.n; r += GS) {
    const double2 a = x[r], b = q.TMP[r];
    acc.x += a.x * b.x + a.y * b.y;  // conj(a) b
    acc.y += a.x * b.y - a.y * b.x;
  }
  return g.sum(acc, q.red);
}

// SME: tr of the d x d matrix whose column-stacked form is v
template <int GS>
__device__ double2 trace_vec(const SdeGroup<GS>& g, const Sde& q, const double2* v) {
  const int d = q.S->d;
  double2 acc = make_double2(0.0, 0.0);
  for (int k = g.rank; k < d; k += GS) {
    const double2 a = v[(int64_t)k * (d + 1)];
    acc.x += a.x;
    acc.y += a.y;
  }
  return g.sum(acc, q.red);
}

// out = drift(x)   (ssystem.pyx:141-154 closed, 227-228 open)
template <int GS>
__device__ void drift(const SdeGroup<GS>& g, const Sde& q, const double2* x, double2* out) {
  const qg_sde& S = *q.S;
  g.sync();
  csr_mv(g, S.l_rp, S.l_col, static_cast<const double2*>(S.l_val), 0, x, out, q.n);
  if (S.open) return;
  for (int i = 0; i < q.m; ++i) {
    const double2 e = expect_m(g, q, i, x);
    g.sync();
    csr_mv(g, S.c_rp, S.c_col, static_cast<const double2*>(S.c_val), (int64_t)i * q.n, x,
           q.TMP, q.n);
    const double2 s1 = cmul2(make_double2(-0.125 * e.x, -0.125 * e.y), e);  // -0.125 * e * e
    const double2 s2 = make_double2(0.5 * e.x, 0.5 * e.y);
    for (int r = g.rank; r < q.n; r += GS) {
      const double2 o = axpy(out[r], s1, x[r]);
      out[r] = axpy(o, s2, q.TMP[r]);
    }
  }
}

// d2[i] = diffusion_i(x) for every i   (ssystem.pyx:156-166 closed, 230-240 open)
template <int GS>
__device__ void diffusion(const SdeGroup<GS>& g, const Sde& q, const double2* x, double2* d2) {
  const qg_sde& S = *q.S;
  for (int i = 0; i < q.m; ++i) {
    double2* out = d2 + (int64_t)i * q.n;
    g.sync();
    csr_mv(g, S.c_rp, S.c_col, static_cast<const double2*>(S.c_val), (int64_t)i * q.n, x, out,
           q.n);
    double2 e;
    if (S.open) {
      g.sync();
      e = trace_vec(g, q, out);
      e = make_double2(-e.x, -e.y);
    } else {
      e = expect_m(g, q, i, x);
      e = make_double2(-0.5 * e.x, -0.5 * e.y);
    }
    for (int r = g.rank; r < q.n; r += GS) out[r] = axpy(out[r], e, x[r]);
  }
}

// One Platen step from X into OUT (_sode.pyx:62-120).
template <int GS>
__device__ void platen_step(const SdeGroup<GS>& g, const Sde& q, const double2* X, double2* OUT,
                            const double* dW, double dt) {
  const int n = q.n, m = q.m;
  const double sqrt_dt = sqrt(dt);
  const double sqrt_dt_inv = 0.25 / sqrt_dt;
  drift(g, q, X, q.F);
  for (int r = g.rank; r < n; r += GS) q.D1[r] = axpy(X[r], dt, q.F[r]);
  diffusion(g, q, X, q.D2);
  for (int r = g.rank; r < n; r += GS) {
    const double2 d1 = q.D1[r];
    OUT[r] = make_double2(d1.x * 0.5, d1.y * 0.5);
    double2 vt = d1;
    for (int i = 0; i < m; ++i) {
      const double2 d2 = q.D2[(int64_t)i * n + r];
      q.VP[(int64_t)i * n + r] = axpy(d1, sqrt_dt, d2);
      q.VM[(int64_t)i * n + r] = axpy(d1, -sqrt_dt, d2);
      vt = axpy(vt, dW[i], d2);
    }
    q.VT[r] = vt;
  }
  drift(g, q, q.VT, q.F);
  for (int r = g.rank; r < n; r += GS) {
    const double2 o = axpy(OUT[r], 0.5 * dt, q.F[r]);
    OUT[r] = axpy(o, 0.5, X[r]);
  }
  for (int i = 0; i < m; ++i) {
    diffusion(g, q, q.VP + (int64_t)i * n, q.D2P);
    diffusion(g, q, q.VM + (int64_t)i * n, q.D2M);
    const double dw = dW[i] * 0.25;
    for (int r = g.rank; r < n; r += GS) {
      double2 o = axpy(OUT[r], 2 * dw, q.D2[(int64_t)i * n + r]);
      for (int j = 0; j < m; ++j) {
        double dw2p, dw2m;
        if (i == j) {
          const double dw2 = sqrt_dt_inv * (dW[i] * dW[j] - dt);
          dw2p = dw2 + dw;
          dw2m = -dw2 + dw;
        } else {
          dw2p = sqrt_dt_inv * dW[i] * dW[j];
          dw2m = -dw2p;
        }
        o = axpy(o, dw2p, q.D2P[(int64_t)j * n + r]);
        o = axpy(o, dw2m, q.D2M[(int64_t)j * n + r]);
      }
      OUT[r] = o;
    }
  }
}

// One Euler-Maruyama step from X into OUT (_sode.pyx:32-55): X + dt drift + sum_i dW_i d2_i.
template <int GS>
__device__ void euler_step(const SdeGroup<GS>& g, const Sde& q, const double2* X, double2* OUT,
                           const double* dW, double dt) {
  drift(g, q, X, q.F);
  diffusion(g, q, X, q.D2);
  for (int r = g.rank; r < q.n; r += GS) {
    double2 o = axpy(X[r], dt, q.F[r]);
    for (int i = 0; i < q.m; ++i) o = axpy(o, dW[i], q.D2[(int64_t)i * q.n + r]);
    OUT[r] = o;
  }
}

constexpr int SDE_PLATEN = 0, SDE_EULER = 1;

template <int GS, int SCHEME>
__device__ void run_trajectory(const SdeGroup<GS>& g, const qg_sde& S, int traj,
                               double2* states, const double* dW, int n_steps, double dt,
                               int64_t work_values, double* red) {
  Sde q;
  q.S = &S;
  q.n = (int)S.n;
  q.m = S.n_sc;
  q.red = red;
  const int64_t n = S.n, m = S.n_sc;
  double2* w = static_cast<double2*>(S.work) + (int64_t)traj * work_values;
  q.F = w;
  q.D1 = w + n;
  q.VT = w + 2 * n;
  q.TMP = w + 3 * n;
  double2* spare = w + 4 * n;  // the other half of the state double buffer
  q.D2 = w + 5 * n;
  q.VP = q.D2 + m * n;
  q.VM = q.VP + m * n;
  q.D2P = q.VM + m * n;
  q.D2M = q.D2P + m * n;
  double2* home = states + (int64_t)traj * n;
  double2* X = home;
  double2* OUT = spare;
  const double* dwt = dW + (int64_t)traj * n_steps * m;
  for (int k = 0; k < n_steps; ++k) {
    if constexpr (SCHEME == SDE_EULER)
      euler_step(g, q, X, OUT, dwt + (int64_t)k * m, dt);
    else
      platen_step(g, q, X, OUT, dwt + (int64_t)k * m, dt);
    g.sync();
    double2* t = X;
    X = OUT;
    OUT = t;
  }
  if (X != home) {  // odd step count: the state ended in the spare
    for (int r = g.rank; r < q.n; r += GS) home[r] = X[r];
  }
}

template <int SCHEME>
__global__ void __launch_bounds__(SDE_BLOCK) sde_cta_kernel(qg_sde S, double2* states,
                                                            const double* __restrict__ dW,
                                                            int n_steps, double dt,
                                                            int64_t work_values) {
  __shared__ double red[2 * SDE_BLOCK / 32];
  const SdeGroup<SDE_BLOCK> g{(int)threadIdx.x};
  run_trajectory<SDE_BLOCK, SCHEME>(g, S, blockIdx.x, states, dW, n_steps, dt, work_values, red);
}

template <int SCHEME>
__global__ void __launch_bounds__(32 * SDE_WARPS) sde_warp_kernel(
    qg_sde S, int n_traj, double2* states, const double* __restrict__ dW, int n_steps, double dt,
    int64_t work_values) {
  const int traj = blockIdx.x * SDE_WARPS + (threadIdx.x >> 5);
  if (traj >= n_traj) return;  // whole warps leave together
  const SdeGroup<32> g{(int)(threadIdx.x & 31)};
  run_trajectory<32, SCHEME>(g, S, traj, states, dW, n_steps, dt, work_values, nullptr);
}

static int check_sde(const qg_sde* S) {
  if (!S) return set_error(QG_ERR_ARG, "null system");
  if (S->n < 1 || S->n >= (int64_t)INT32_MAX / (QG_MAX_COPS + 1))
    return set_error(QG_ERR_ARG, "state length out of range");
  if (S->n_sc < 1 || S->n_sc > QG_MAX_COPS) return set_error(QG_ERR_ARG, "n_sc out of range");
  if (S->open != 0 && S->open != 1) return set_error(QG_ERR_ARG, "open must be 0 or 1");
  if (S->open && (int64_t)S->d * S->d != S->n)
    return set_error(QG_ERR_ARG, "SME: the state length must be d*d");
  if (!S->open && S->d != S->n) return set_error(QG_ERR_ARG, "SSE: the state length must be d");
  if (!S->l_rp || !S->l_col || !S->l_val || !S->c_rp || !S->c_col || !S->c_val || !S->work)
    return set_error(QG_ERR_ARG, "null operator or workspace");
  if (!S->open && (!S->m_rp || !S->m_col || !S->m_val))
    return set_error(QG_ERR_ARG, "SSE needs the expectation operators");
  return QG_OK;
}

template <int SCHEME>
static int launch_sde(const qg_sde* S, int32_t n_traj, void* states, const double* dW,
                      int32_t n_steps, double dt, void* stream) {
  int rc = check_sde(S);
  if (rc) return rc;
  if (n_traj < 0 || n_steps < 0 || !(dt > 0.0)) return set_error(QG_ERR_ARG, "bad launch");
  if (n_traj == 0 || n_steps == 0) return QG_OK;
  if (!states || !dW) return set_error(QG_ERR_ARG, "null states or noise");
  const int64_t wv = (5 + 5 * (int64_t)S->n_sc) * S->n;
  if (S->n <= SDE_WARP_MAX_N) {
    sde_warp_kernel<SCHEME><<<(n_traj + SDE_WARPS - 1) / SDE_WARPS, 32 * SDE_WARPS, 0,
                              (cudaStream_t)stream>>>(*S, n_traj, static_cast<double2*>(states),
                                                      dW, n_steps, dt, wv);
    return check_launch("sde_warp_kernel");
  }
  sde_cta_kernel<SCHEME><<<n_traj, SDE_BLOCK, 0, (cudaStream_t)stream>>>(
      *S, static_cast<double2*>(states), dW, n_steps, dt, wv);
  return check_launch("sde_cta_kernel");
}

}  // namespace qg

using namespace qg;

extern "C" int64_t qg_sde_work_values(int64_t n, int32_t n_sc) {
  return (5 + 5 * (int64_t)n_sc) * n;
}

extern "C" int qg_sde_platen(const qg_sde* S, int32_t n_traj, void* states, const double* dW,
                             int32_t n_steps, double dt, void* stream) {
  return launch_sde<SDE_PLATEN>(S, n_traj, states, dW, n_steps, dt, stream);
}

extern "C" int qg_sde_euler(const qg_sde* S, int32_t n_traj, void* states, const double* dW,
                            int32_t n_steps, double dt, void* stream) {
  return launch_sde<SDE_EULER>(S, n_traj, states, dW, n_steps, dt, stream);
}
