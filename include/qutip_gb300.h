/*
 * qutip_gb300 -- C ABI of the GB300 (sm_103a) time-evolution hot path.
 *
 * Every entry point takes plain device pointers, sizes and a cudaStream_t
 * (passed as void*), returns 0 on success or a negative QG_ERR_* code, and never
 * allocates or frees caller memory; qg_last_error() gives the message of the
 * last failure on the calling thread.  Buffers are owned by the caller (the
 * Python host layer keeps them in torch tensors).
 *
 * Each declaration names the reference function it replaces (paths relative to
 * the QuTiP source tree).
 */
#ifndef QUTIP_GB300_H
#define QUTIP_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QG_OK 0
#define QG_ERR_ARG (-1)         /* bad argument: shape, size or pointer (reference: ValueError) */
#define QG_ERR_CUDA (-2)        /* CUDA runtime error */
#define QG_ERR_UNSUPPORTED (-3) /* dtype / option not supported (reference: TypeError) */

#define QG_MAX_GROUPS 8   /* coefficient groups (QobjEvo terms after merging) per operator */
#define QG_MAX_EOPS 32    /* operators per expect launch */
#define QG_MAX_COPS 64    /* collapse operators of one matrix-free Lindblad generator */

typedef enum { QG_C128 = 0, QG_C64 = 1 } qg_dtype;

/* Integrator status codes, same values as Status in
 * qutip/solver/integrator/explicit_rk.pxd:5-12. */
typedef enum {
  QG_AT_FRONT = 2,
  QG_INTERPOLATED = 1,
  QG_NORMAL = 0,
  QG_TOO_MUCH_WORK = -1,
  QG_DT_UNDERFLOW = -2,
  QG_OUTSIDE_RANGE = -3,
  QG_NOT_INITIATED = -4,
  QG_NORM_SEARCH_FAILED = -5, /* jump-time search exhausted (qutip/solver/mcsolve.py:363-367) */
  QG_TIMEOUT = -6,            /* cancelled through the host-visible cancel flag */
  QG_JUMP_OVERFLOW = -7,      /* more jumps than the batch's max_jumps */
  QG_BAD_ITEM = -8            /* item not run: bad system index, state longer than max_n,
                                 or a group count outside 1..QG_MAX_GROUPS */
} qg_status;

/* A sum of CSR matrices with time-dependent coefficients,
 *   A(t) = sum_g c_g(t) A_g,
 * the device form of a QobjEvo (qutip/core/cy/qobjevo.pyx:189-245) whose terms
 * were merged per coefficient.  Two layouts of the row pointers:
 *   QG_LAYOUT_GROUP_MAJOR: group g's row r spans
 *       [row_ptr[g*(n_rows+1)+r], row_ptr[g*(n_rows+1)+r+1]) of col/val;
 *   QG_LAYOUT_ROW_MAJOR: the entries of row r are stored contiguously, group by
 *       group: group g of row r spans [row_ptr[r*G+g], row_ptr[r*G+g+1]) and
 *       row_ptr[n_rows*G] is the number of entries.
 * Launch shape: lanes = threads per row (power of two, 1..32).  n_tiles > 0
 * selects the shared-memory staged kernel (ROW_MAJOR only): tile t covers rows
 * [tile_row[t], tile_row[t+1]) holding at most tile_nnz - 8 entries and at most
 * QG_TILE_ROWS rows; col, val and row_ptr must then be readable for 8 entries
 * past their end (bulk copies are rounded to 16-byte units).
 * QG_LAYOUT_SLICED (sliced ELLPACK, 32-row slices): slice s holds rows
 *   [32 s, 32 s + 32); row_ptr[s] is the entry offset of the slice (n_slices + 1
 *   values, n_slices = n_tiles) and tile_row[s*G + g] the width of group g in that
 *   slice; entry j of group g of the row at lane l sits at
 *   row_ptr[s] + 32 * (sum_{g'<g} width_g') + 32 j + l.  Padding entries have
 *   value 0 and a valid column.  One thread per row; lanes and tile_nnz unused.
 * QG_LAYOUT_SLICED_DICT (dictionary-coded sliced ELLPACK, for operators whose entries
 *   repeat a few (column - row, value) pairs, as Kronecker-structured Liouvillians do):
 *   32-row slices as above, but every stored entry is a code into its group's table:
 *   code k of group g stands for column row + dict_off[dict_start[g] + k] and value
 *   val[dict_start[g] + k] (val holds the tables, lanes = their total length, at most
 *   QG_DICT_MAX); code 0 of every group is padding (offset 0, value 0).  col points to
 *   the codes, tile_nnz bytes each (1 or 2).  Each group has its own code section:
 *   row_ptr[g*(n_tiles+1) + s] is the code offset of slice s of group g (a multiple of
 *   128), tile_row[s*G + g] its width w (the longest row; the section holds 4*ceil(w/4)
 *   codes per lane), and codes are stored four per lane: entries 4q..4q+3 of lane l of
 *   the slice at row_ptr[...] + 128 q + 4 l + (0..3).  Columns are clamped into
 *   [0, n_cols), so no code can address outside x.
 * QG_LAYOUT_SLICED_DICT_RI (complex128 only): QG_LAYOUT_SLICED_DICT with the real and the
 *   imaginary part of every entry coded separately, so that a code costs two FP64
 *   multiply-adds instead of four.  Table entry t stands for column
 *   row + (dict_off[t] >> 1); with the low bit of dict_off[t] clear it is the real part a
 *   of an entry and val[t] = (a, a), with it set an imaginary part i a and
 *   val[t] = (-a, a).  The product is (val.re * p, val.im * q) with (p, q) = (x.re, x.im),
 *   or (x.im, x.re) for an imaginary part.  A complex entry occupies two codes.
 * Coefficient programs are the bytecode of qutip_gb300/coefficients.py;
 * coef_code == NULL means every c_g = 1. */
#define QG_LAYOUT_GROUP_MAJOR 0
#define QG_LAYOUT_ROW_MAJOR 1
#define QG_LAYOUT_SLICED 2
#define QG_LAYOUT_SLICED_DICT 3
#define QG_LAYOUT_SLICED_DICT_RI 4
#define QG_DICT_MAX 4096
#define QG_TILE_ROWS 512
typedef struct qg_csr_groups {
  int64_t n_rows;
  int64_t n_cols;
  int32_t n_groups;
  int32_t dtype; /* qg_dtype of val */
  int32_t layout;
  int32_t lanes;
  int32_t n_tiles;
  int32_t tile_nnz; /* 2048 or 4096 */
  const int32_t* row_ptr;
  const int32_t* col;
  const void* val;
  const int32_t* tile_row;
  const int32_t* coef_code;
  const int32_t* coef_start; /* [n_groups+1] */
  const double* coef_consts; /* complex constants as (re, im) pairs */
  const int32_t* dict_off;   /* dictionary layouts: column - row of each table entry */
  const int32_t* dict_start; /* dictionary layouts: [n_groups+1] table bounds */
} qg_csr_groups;

/* Dia matrix in the reference's layout (qutip/core/data/dia.pxd:17-38):
 * data[d * n_cols + col] is the entry (col - offsets[d], col). */
typedef struct qg_dia {
  int64_t n_rows;
  int64_t n_cols;
  int32_t n_diags;
  int32_t dtype;
  const int32_t* offsets;
  const void* data;
} qg_dia;

/* The Lindblad generator applied to vec(rho) without forming its d^2 x d^2
 * superoperator (the reference's matrix form,
 * qutip/core/cy/lindblad_matrix_form.pyx:105-204, in its full non-Hermitian branch):
 *   L[rho] = A rho + rho A^dag + sum_i |f_i(t)|^2 C_i rho C_i^dag,
 *   A(t) = sum_g a_g(t) A_g = -i H_nh(t),  H_nh = H - (i/2) sum_i |f_i|^2 C_i^dag C_i,
 * where vec(rho) is the column-major d*d vector (rho[r, c] at r + c*d, the F order of
 * qutip's Dense) and the i-th collapse operator is f_i(t) C_i.
 * Storage ("ELL" blocks: entry j of row r of a block of width W at base + j*d + r, so
 * that consecutive rows are consecutive in memory; padding entries have value 0 and a
 * valid column):
 *   A_g:  its diagonal at a_diag[g*d + r] and its off-diagonal entries in an ELL
 *         block of width a_width[g]; the blocks of g = 0..n_groups-1 follow one
 *         another in a_col / a_val (block g starts at d * sum_{g'<g} a_width[g']);
 *         the widths are held in this struct (host memory);
 *   C_i:  the first n_diag_cops are diagonal, C_i[r,r] at c_diag[i*d + r]; the other
 *         n_cops - n_diag_cops are ELL blocks of width c_width[i - n_diag_cops] in
 *         c_col / c_val, one after another.
 * Constant diagonal part: d_const (d*d entries in dtype, may be NULL) holds
 *   D0(r, c) = sum_{g in const} A_g[r,r] + conj(A_g[c,c])
 *            + sum_{i < n_const_diag} C_i[r,r] conj(C_i[c,c])
 * at r + c*d for the groups whose bit in a_diag_const is set (coefficient 1, folded
 * in D0) and the first n_const_diag diagonal collapse operators (coefficient 1); the
 * other diagonal parts are evaluated per element.  With d_const NULL, a_diag_const
 * and n_const_diag must be 0.
 * Coefficient programs: a_g for the groups of A, f_i for the collapse operators in
 * the order above (NULL code: all 1).  1 <= n_groups <= QG_MAX_GROUPS,
 * 0 <= n_diag_cops <= n_cops <= QG_MAX_COPS, d*d < 2^31, ELL blocks < 2^31 entries. */
typedef struct qg_lindblad {
  int64_t d;
  int32_t dtype;
  int32_t n_groups;
  int32_t n_diag_cops;
  int32_t n_cops;
  int32_t a_diag_const; /* bit g: the diagonal of A_g is folded into d_const */
  int32_t n_const_diag; /* leading diagonal collapse operators folded into d_const */
  int32_t hermitian;    /* 1: rho is Hermitian; elements r >= c are evaluated and mirrored
                           (out[c + r d] = conj(out[r + c d]), real diagonal), the reference's
                           assume_hermitian_state branch (lindblad_matrix_form.pyx:171-188) */
  int32_t reserved;     /* 0 */
  int32_t a_width[QG_MAX_GROUPS];
  int32_t c_width[QG_MAX_COPS];
  const void* d_const;
  const void* a_diag;
  const int32_t* a_col;
  const void* a_val;
  const void* c_diag;
  const int32_t* c_col;
  const void* c_val;
  const int32_t* a_coef_code;
  const int32_t* a_coef_start;
  const double* a_coef_consts;
  const int32_t* c_coef_code;
  const int32_t* c_coef_start;
  const double* c_coef_consts;
} qg_lindblad;

/* Dense small-dimension bucket (d <= QG_DENSE_MAX_D): the Lindblad generator with
 * dense operators, L(t)[X] = A X + X A^dag + sum_i |f_i(t)|^2 C_i X C_i^dag with
 * A = sum_g a_g(t) A_g = -i H_nh, applied as GEMMs on the tensor cores (TF32 split into
 * hi + lo parts, FP32 accumulation).  Operators are complex64, row-major:
 * A_g[m][k] at a + (g*d + m)*d + k, C_i[m][k] at c + (i*d + m)*d + k.  Coefficient
 * programs as in qg_lindblad (NULL code: all 1).  One CTA per 16 columns of the
 * result; no workspace. */
#define QG_DENSE_MAX_D 128
typedef struct qg_dense_lindblad {
  int32_t d;
  int32_t n_groups;
  int32_t n_cops;
  int32_t reserved; /* 0 */
  const void* a;
  const void* c;
  const int32_t* a_coef_code;
  const int32_t* a_coef_start;
  const double* a_coef_consts;
  const int32_t* c_coef_code;
  const int32_t* c_coef_start;
  const double* c_coef_consts;
} qg_dense_lindblad;

/* Buffers of one explicit Runge-Kutta step.  The state (y_prev, y_front) may be
 * complex128 while the stages (k, ytmp) are complex64 ("mixed" form): the
 * state update of each accepted step and the error norm stay in FP64, the stage
 * combinations run in FP32 from y_prev_s, a complex64 copy of y_prev that stage 9
 * refreshes (y_front_s) together with y_front.  When state and stages share a
 * dtype, y_prev_s / y_front_s are unused (may be NULL). */
typedef struct qg_rk_buffers {
  int64_t n;
  int32_t state_dtype;
  int32_t stage_dtype;
  const void* y_prev;    /* [n] state_dtype */
  void* y_front;         /* [n] state_dtype */
  const void* y_prev_s;  /* [n] stage_dtype, mixed form only */
  void* y_front_s;       /* [n] stage_dtype, mixed form only */
  void* k;               /* [16 * n] stage_dtype, k_j at k + j*n */
  void* ytmp;            /* [2 * n] stage_dtype, stage inputs (ping-pong) */
  double* scratch;       /* [qg_scratch_doubles()] per-block partial sums */
  unsigned int* counter; /* one word, zero before the first launch; left zero */
  double* result;        /* one double: WRMS error of the step */
} qg_rk_buffers;

/* A state given lazily as base + sum_j f_j k_j (an interpolated Runge-Kutta
 * output, qutip/solver/integrator/explicit_rk.pyx:412-430); n_k = 0 means base. */
typedef struct qg_state_view {
  int64_t n;
  int32_t base_dtype;
  int32_t k_dtype;
  const void* base;
  const void* k; /* k_j at k + j*n */
  int32_t n_k;
  int32_t pad_;
  double f[16];
} qg_state_view;

/* ---- library ---------------------------------------------------------- */
int qg_version(void);
const char* qg_last_error(void);
/* sizeof of the ABI structs, in this order: qg_csr_groups, qg_dia, qg_rk_buffers,
 * qg_state_view, qg_batch_system, qg_batch_item, qg_batch (host only; lets a
 * binding check its struct layouts).  Returns the number written. */
int qg_abi_sizes(int64_t* out, int n);
/* Number of doubles the scratch buffer of qg_rk_buffers / reductions needs. */
int64_t qg_scratch_doubles(void);
/* Copy the compiled-in Vern7 tableau (host memory, no GPU needed):
 * a[16*16], b[10], c[16], e[10], bi[16*7]; replaces
 * qutip/solver/integrator/verner7efficient.py:10-333. */
int qg_vern7_tableau(double* a, double* b, double* c, double* e, double* bi);

/* ---- matvec ------------------------------------------------------------- */
/* y = alpha * sum_g c_g(t) A_g x + beta * y, vectors in A->dtype, FP64
 * accumulation for complex128 and FP32 for complex64.  Replaces _matmul_csr_vector
 * (qutip/core/data/src/matmul_csr_vector.cpp:17-54, scalar form :107-149) as
 * driven by QobjEvo.matmul_data (qutip/core/cy/qobjevo.pyx:1103-1116) and
 * matmul_csr_dense_dense (qutip/core/data/matmul.pyx:226-272). */
int qg_spmv_csr(const qg_csr_groups* A, double t, const void* x, void* y, double alpha_re,
                double alpha_im, double beta_re, double beta_im, void* stream);

/* Y = alpha * A(t) X + beta * Y for n_vec column vectors stored with leading
 * dimension ld (F order): one operator read serves all columns.  Replaces the
 * per-column loop of matmul_csr_dense_dense (qutip/core/data/matmul.pyx:255-270)
 * and _matmul_csr_dense_c_order (qutip/core/data/src/matmul_csr_dense.cpp:20-70). */
int qg_spmm_csr(const qg_csr_groups* A, double t, const void* X, void* Y, int64_t n_vec,
                int64_t ld, double alpha_re, double alpha_im, double beta_re, double beta_im,
                void* stream);

/* y = alpha * A x + beta * y for a Dia matrix.  Replaces matmul_dia_dense_dense
 * (qutip/core/data/matmul.pyx:429-507) and _matmul_diag_vector
 * (qutip/core/data/src/matmul_diag_vector.cpp:13-39). */
int qg_spmv_dia(const qg_dia* A, const void* x, void* y, double alpha_re, double alpha_im,
                double beta_re, double beta_im, void* stream);

/* ---- Vern7 step ----------------------------------------------------------- */
/* One Runge-Kutta stage fused with the next stage's combination:
 *   k_s = A(t_prev + c_s dt) x_s,  x_0 = y_prev (y_prev_s in the mixed form),
 *   x_s = ytmp[s & 1];
 *   s in 0..8, 10..14:  ytmp[(s+1) & 1] = y_prev + sum_{j<=s} (dt a[s+1][j]) k_j
 *   s == 9:  y_front = y_prev + sum_j (dt b_j) k_j and
 *            result = sqrt(mean((|sum_j dt e_j k_j| / (atol + rtol |y_front|))^2))
 * Replaces _compute_step / _accumulate / _error / _prep_dense_out
 * (qutip/solver/integrator/explicit_rk.pyx:358-410) with wrmn_error_dense
 * (qutip/core/data/ode.pyx:27-52) and iadd_dense (qutip/core/data/add.pyx:203-219). */
int qg_vern7_stage(const qg_csr_groups* A, const qg_rk_buffers* B, int stage, double t_prev,
                   double dt, double atol, double rtol, void* stream);

/* y = alpha * L(t)[x] + beta * y for the matrix-free Lindblad generator; x and y
 * are vec(rho) of length d*d in L's dtype.  Replaces LindbladMatrixForm.matmul_data
 * (qutip/core/cy/lindblad_matrix_form.pyx:105-204). */
int qg_lindblad_apply(const qg_lindblad* L, double t, const void* x, void* y, double alpha_re,
                      double alpha_im, double beta_re, double beta_im, void* stream);

/* qg_vern7_stage with the matrix-free Lindblad generator in place of A(t): one
 * Vern7 stage of mesolve with options matrix_form=True (qutip/solver/mesolve.py:251-266);
 * B->n = d*d. */
int qg_lindblad_stage(const qg_lindblad* L, const qg_rk_buffers* B, int stage, double t_prev,
                      double dt, double atol, double rtol, void* stream);

/* y = alpha * L(t)[x] + beta * y for the dense generator; x, y complex64 vec(rho) of
 * length d*d.  Replaces LindbladMatrixForm.matmul_data
 * (qutip/core/cy/lindblad_matrix_form.pyx:105-204, full branch) for small dense systems;
 * one CTA per application, tcgen05 tensor-core GEMMs. */
int qg_dense_lindblad_apply(const qg_dense_lindblad* L, double t, const void* x, void* y,
                            double alpha_re, double alpha_im, double beta_re, double beta_im,
                            void* stream);

/* qg_vern7_stage with the dense generator: complex64 stages (B->stage_dtype = QG_C64),
 * the state complex128 (mixed form) or complex64; B->n = d*d. */
int qg_dense_lindblad_stage(const qg_dense_lindblad* L, const qg_rk_buffers* B, int stage,
                            double t_prev, double dt, double atol, double rtol, void* stream);

/* Stochastic Schrodinger / master equations (ssesolve / smesolve), the reference's
 * explicit Platen scheme (qutip/solver/sode/_sode.pyx:58-120) on the systems of
 * qutip/solver/sode/ssystem.pyx:119-250:
 *   SSE (open = 0, state psi, n = d):  drift = L psi + sum_i (-e_i^2/8 psi + e_i/2 C_i psi),
 *     L = -i H - 1/2 sum_i C_i^dag C_i, e_i = <psi| M_i |psi> with M_i = C_i + C_i^dag;
 *     diffusion_i = C_i psi - e_i/2 psi.
 *   SME (open = 1, state vec(rho), n = d*d): drift = L rho (L the Liouvillian of H, sc_ops
 *     and c_ops), diffusion_i = C_i rho - tr(C_i rho) rho with C_i = spre(c_i) + spost(c_i^dag).
 * Operators are complex128 CSR with 32-bit indices; the n_sc stochastic operators (and the
 * SSE expectation operators) are stacked by rows: block i holds rows i*n .. i*n + n - 1. */
typedef struct qg_sde {
  int64_t n;        /* state length */
  int32_t open;     /* 0: SSE (ket), 1: SME (vec(rho), column-stacked) */
  int32_t n_sc;     /* stochastic operators (1..QG_MAX_COPS) */
  int32_t d;        /* Hilbert-space dimension */
  int32_t reserved; /* 0 */
  const int32_t* l_rp;
  const int32_t* l_col;
  const void* l_val;
  const int32_t* c_rp;
  const int32_t* c_col;
  const void* c_val;
  const int32_t* m_rp;  /* SSE only (NULL for SME) */
  const int32_t* m_col;
  const void* m_val;
  void* work;       /* n_traj * qg_sde_work_values(n, n_sc) complex128 values */
} qg_sde;

/* Workspace of one trajectory, in complex128 values. */
int64_t qg_sde_work_values(int64_t n, int32_t n_sc);

/* n_steps Platen steps of dt for each of n_traj trajectories (one CTA each): states holds
 * n_traj complex128 states of length n (updated in place); dW holds the Wiener increments,
 * n_traj x n_steps x n_sc doubles (trajectory-major), as the reference's Wiener.dW draws
 * them.  Replaces PlatenSODE.integrate / _sode.Platen.run (sode.py:151-173). */
int qg_sde_platen(const qg_sde* S, int32_t n_traj, void* states, const double* dW,
                  int32_t n_steps, double dt, void* stream);

/* The same with the Euler-Maruyama scheme (EulerSODE, qutip/solver/sode/itotaylor.py:12-26;
 * steps in qutip/solver/sode/_sode.pyx:32-55): x + dt drift(x) + sum_i dW_i diffusion_i(x). */
int qg_sde_euler(const qg_sde* S, int32_t n_traj, void* states, const double* dW,
                 int32_t n_steps, double dt, void* stream);

/* Non-zero when a kernel of this library gave up a bounded wait on the current
 * device (the result of that launch is invalid); reading clears the flag. */
int qg_device_fault(void);

/* out = base + sum_{j<n_k} f_j k_j (out in out_dtype).  Replaces _accumulate
 * and _interpolate_step (qutip/solver/integrator/explicit_rk.pyx:412-437). */
int qg_rk_combine(const qg_state_view* v, void* out, int out_dtype, void* stream);

/* *result = sum |x_i|^2 in FP64 (deterministic two-level reduction through
 * scratch/counter).  Replaces frobenius_dense / l2 (qutip/core/data/norm.pyx:127-135). */
int qg_norm2(const void* x, int dtype, int64_t n, double* scratch, unsigned int* counter,
             double* result, void* stream);

/* ---- expectation values --------------------------------------------------- */
/* For a column-stacked density matrix rho (d x d) given by a state view:
 * out[2g], out[2g+1] = tr(op_g rho) for each group g of ops (each group is one
 * d x d operator, coefficients ignored) and out[2G], out[2G+1] = tr(rho), FP64.
 * Replaces _expect_csr_dense_dm (qutip/core/data/expect.pyx:146-158) and
 * expect_super_csr_dense (:223-236) as used by Result.add for e_ops. */
int qg_expect_dm(const qg_csr_groups* ops, int64_t d, const qg_state_view* rho, double* out,
                 void* stream);

/* out[2g..] = <psi|op_g|psi>, out[2G..] = <psi|psi>.  Replaces
 * _expect_csr_dense_ket (qutip/core/data/expect.pyx:133-144). */
int qg_expect_ket(const qg_csr_groups* ops, const qg_state_view* psi, double* out, void* stream);

/* ---- batched, persistent solves ----------------------------------------- */
/* One system of a batch.  Its generator is a row-major grouped CSR in the
 * operator pools (rows r: row_ptr[rp_off + r*G + g], absolute entry offsets);
 * kind 0 = master equation on a column-stacked density matrix (n = d*d),
 * kind 1 = Monte-Carlo trajectory of a ket (n = d) with the effective
 * non-Hermitian generator and n_cops collapse operators. */
typedef struct qg_batch_system {
  int32_t n;         /* state length */
  int32_t d;         /* Hilbert-space dimension */
  int32_t n_groups;  /* generator coefficient groups */
  int32_t n_eops;    /* e_ops (CSR d x d, group-major, one group each) */
  int64_t rp_off;    /* generator row pointers in op_rp */
  int64_t coef_off;  /* n_groups+1 program starts in coef_start (-1: constant generator) */
  int64_t eop_rp_off;  /* e_op e row r: eop_rp[eop_rp_off + e*(d+1) + r] */
  int64_t cop_rp_off;  /* collapse op c row r: cop_rp[cop_rp_off + c*(d+1) + r] */
  int64_t tlist_off; /* n_out output times in tlist */
  int32_t n_out;
  int32_t kind;
  int32_t n_cops;
  int32_t nsteps;    /* maximum steps per output interval (reference option nsteps) */
  double atol, rtol;
  int64_t cop_coef_off; /* n_cops program starts in coef_start, collapse operator c being
                           f_c(t) C_c (mcsolve.py:168-170 wraps every c_op in a QobjEvo);
                           -1: constant collapse operators */
} qg_batch_system;

/* One unit of work: a system solved from an initial state, or one trajectory
 * of an MC system with its own PCG64 stream (state and increment as 128-bit
 * pairs, numpy's PCG64 state after seeding). */
typedef struct qg_batch_item {
  int32_t system;
  int32_t pad_;
  int64_t y0_off;   /* initial state (complex128) in y0 */
  int64_t out_off;  /* n_out * (n_eops+1) complex128 results in out */
  uint64_t rng_state_hi, rng_state_lo, rng_inc_hi, rng_inc_lo;
  /* improved sampling (qutip/solver/mcsolve.py:245-279): the first jump target is
   * random() * (1 - jump_prob_floor) + jump_prob_floor, so a trajectory with a floor
   * equal to the no-jump probability always jumps; 0 for ordinary trajectories.
   * Later targets (after each jump) are drawn without the floor (mcsolve.py:405). */
  double jump_prob_floor;
} qg_batch_item;

typedef struct qg_batch {
  int32_t n_systems;
  int32_t n_items;
  int32_t dtype;     /* generator / stage dtype; the state is complex128 */
  int32_t max_n;     /* largest state length (workspace per slot) */
  const qg_batch_system* systems; /* device */
  const qg_batch_item* items;     /* device; processed in this order */
  const int32_t* op_rp;
  const int32_t* op_col;
  const void* op_val;
  const int32_t* coef_code;
  const int32_t* coef_start;
  const double* coef_consts;
  const int32_t* eop_rp;
  const int32_t* eop_col;
  const double* eop_val;  /* complex128 pairs */
  const int32_t* cop_rp;
  const int32_t* cop_col;
  const double* cop_val;  /* complex128 pairs */
  const double* tlist;
  const double* y0;       /* complex128 pairs */
  double* out;            /* e_op values (complex128 pairs); the last slot per output is
                             tr(rho) (kind 0) or <psi|psi> (kind 1, after normalisation) */
  int32_t* status;        /* [n_items * 4]: qg_status, steps, rhs calls, jumps */
  double* jump_t;         /* [n_items * max_jumps] */
  int32_t* jump_which;    /* [n_items * max_jumps] */
  int32_t max_jumps;
  int32_t n_slots;        /* groups (warps or CTAs, see `group`); each owns one slot */
  void* work;             /* n_slots * qg_batch_slot_bytes(max_n, dtype) bytes */
  unsigned int* queue;    /* four words, zero before the launch; words 0-1 are left zero;
                             word 2 becomes non-zero if an operator-staging wait gave up
                             (the launch then read the operator from global memory) */
  const volatile int32_t* cancel; /* optional host-visible flag; non-zero stops all items */
  int64_t* progress;      /* optional [n_slots]: (item << 32) | output index of each slot */
  double* debug;          /* optional [n_slots * 64]: last trajectory-loop states per slot */
  int32_t norm_steps;     /* MC options (qutip/solver/mcsolve.py:449-466) */
  int32_t group;          /* QG_GROUP_*: threads per item */
  double norm_t_tol, norm_tol, norm_min_step, mc_corr_eps;
  /* Operator staging: when the launch has one system, its generator's row
   * pointers (stage_op_rp words) and entries (stage_op_entries) can be copied once
   * per CTA into shared memory (bulk async copies, mbarrier completion) and read
   * from there; 0 = read from global memory.  Warp and CTA groups only. */
  int64_t stage_op_entries;
  int32_t stage_op_rp;
  int32_t pad2_;
} qg_batch;

/* Threads per item of the batched solver: one warp, one 256-thread CTA, a
 * cluster of 8 such CTAs (on 8 SMs, reductions through distributed shared
 * memory), or the default (a warp when max_n <= 2048, else a CTA). */
#define QG_GROUP_AUTO 0
#define QG_GROUP_WARP 1
#define QG_GROUP_CTA 2
#define QG_GROUP_CLUSTER 3
#define QG_GROUP_CTA128 4 /* one 128-thread CTA per item (half the replicated control) */

/* Workspace bytes of one slot. */
int64_t qg_batch_slot_bytes(int64_t max_n, int dtype);
/* Resident CTAs (useful n_slots) on the current device for this max_n / dtype;
 * negative QG_ERR_* on failure. */
int qg_batch_max_slots(int64_t max_n, int dtype);
/* Resident groups (warps for QG_GROUP_WARP, CTAs for QG_GROUP_CTA, clusters for
 * QG_GROUP_CLUSTER, warps or CTAs for QG_GROUP_AUTO) on the current device: the
 * useful n_slots for that group shape. */
int qg_batch_group_slots(int64_t max_n, int dtype, int group);
/* Resident groups for this launch description (max_n, dtype, group and operator
 * staging of *B): the useful n_slots. */
int qg_batch_launch_slots(const qg_batch* B);
/* Shared-memory bytes per CTA of this launch (stage inputs and staged operator);
 * 0 when nothing is staged. */
int64_t qg_batch_smem_bytes(const qg_batch* B);

/* Solve every item of the batch in one persistent launch: each CTA takes items
 * from an atomic queue and runs the adaptive Vern7 integration of
 * Explicit_RungeKutta (qutip/solver/integrator/explicit_rk.pyx:278-467) with
 * its own step size, writing expectation values at the output times as
 * Result.add does (qutip/solver/solver_base.py:138-157, qutip/core/expect.py:91).
 * kind-1 items run MCIntegrator's jump loop (qutip/solver/mcsolve.py:286-406):
 * norm check after each step, log-ratio bisection of the jump time on the
 * dense output, collapse choice and PCG64 draws in the reference's order. */
int qg_batch_vern7(const qg_batch* B, void* stream);

/* Size of the static workspace of qg_batch_vern7_noalloc (16 MiB per GPU). */
#define QG_NOALLOC_WORK_BYTES (16u << 20)

/* qg_batch_vern7 without any allocation -- no counterpart in the reference.
 * For callers that cannot allocate device memory: a host framework that hands
 * this library only pointers from its own memory pool and forbids allocations
 * outside it, or a latency-critical service loop that must not take the
 * synchronisation of cudaMalloc/cudaFree.  The caller still passes every input
 * and output of qg_batch (pools, out, status, jump buffers); B->work, B->queue
 * and B->n_slots are ignored.  The workspace is a 16 MiB static device array
 * (QG_NOALLOC_WORK_BYTES) that every GPU using the library holds until the
 * process exits; batches whose single slot (qg_batch_slot_bytes(max_n, dtype))
 * does not fit are rejected with QG_ERR_ARG, and the number of concurrent items
 * is what fits.  The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress, with that device current), so make that first call
 * before any stream capture.  All calls share the array and its queue words:
 * calls that overlap on the GPU (different streams, or different host threads)
 * race and corrupt each other; serialise them.  No cudaMalloc, cudaFree or
 * allocating library routine is called.  The device address is kept for the life
 * of the process: resetting the device (cudaDeviceReset) after the first call on it
 * is not supported. */
int qg_batch_vern7_noalloc(const qg_batch* B, void* stream);

/* After qg_batch_vern7_noalloc on this device and stream: 1 if a CTA gave up its
 * bounded wait for the bulk copy of the staged operator (it then read the operator
 * from global memory, so results stay correct but the launch ran slower than
 * planned), 0 if not, negative on error.  The flag lives in the static queue words
 * that the next call clears, so read it before the next call.  Synchronises the
 * stream; allocates nothing. */
int qg_batch_noalloc_staging_fault(void* stream);

#ifdef __cplusplus
}
#endif
#endif /* QUTIP_GB300_H */
