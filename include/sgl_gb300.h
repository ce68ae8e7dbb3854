/*
 * sgl_gb300.h -- C ABI of the GB300 (sm_103a) engine for the hot path of the stochastic
 * weak-lensing magnification PDF: the compensated compound-Poisson characteristic exponent
 * ln Phi(k_kappa, k_gamma) of a binned lens population, its xi_lin (gauss) clustering term,
 * and the Hankel/Fourier inversion to dP/dln(mu).
 *
 * Every entry point takes plain host pointers and sizes (no framework types), returns an
 * sgl_status, and is synchronous with respect to the host on the context's own CUDA stream.
 * A context is re-entrant but must not be shared by two host threads at once.
 *
 * Each function names the reference (sgl_analytic v0.2.0, src/sgl_analytic/) interface it
 * replaces.  The package's own host layer (sgl_analytic_gb300/_lib.py) binds it with ctypes.
 */
#ifndef SGL_GB300_H
#define SGL_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SGL_ABI_VERSION 2

typedef struct sgl_ctx sgl_ctx;

/* Status codes.  The Python layer maps SGL_ERR_VALUE to ValueError and SGL_ERR_NONFINITE to
 * RuntimeError, the reference's exception types for bad input (api.py:14-22,
 * pipeline.py:144-164) and non-finite output (api.py:73-74). */
typedef enum {
    SGL_OK = 0,
    SGL_ERR_VALUE = 1,        /* invalid argument (size, NaN, ordering) */
    SGL_ERR_CUDA = 2,         /* CUDA runtime error; see sgl_last_error */
    SGL_ERR_NONFINITE = 3,    /* a result was NaN / Inf */
    SGL_ERR_STATE = 4,        /* call order (e.g. lnphi before set_cells) */
    SGL_ERR_UNSUPPORTED = 5   /* configuration outside the implemented path */
} sgl_status;

/* Arithmetic of the Lambda evaluation and of the inversion. */
typedef enum {
    SGL_FP64 = 0,   /* FP64 throughout: parity path, max|d lnPhi| <= 1e-10 vs the reference */
    SGL_MIXED = 1   /* float-float phase with exact reduction, FP32 sin/cos/J0, SIMT GEMMs with
                       compensated blocked accumulation and float-float split-K combines, the gauss
                       xi term on tcgen05 (TF32 hi/lo); the k-reach probes sum FP32 terms in FP64.
                       Bars: PDF L1 <= 1e-4, tail relative error <= 1e-3.  sgl_pdf evaluates ln Phi
                       in FP64 for populations of at most 4096 cells (few heavy cells: FP32 rounding
                       of single terms does not average out) */
} sgl_precision;

/* Options of the inversion; defaults = pipeline.run's gauss chain (pipeline.py:221-239). */
typedef struct {
    int precision;        /* sgl_precision for Lambda and the transforms */
    int tail_box;         /* 1: widen the box to kappa 0.99, gamma 0.8 (sgl_full.py:33-36) */
    double phi_tol;       /* |Phi| at the k-reach cut (pipeline default 1e-8) */
    int n_xi_wide;        /* normalisation / moment grid points (500 for gauss) */
    int n_k_int;          /* points per constant-mu path (2400) */
    double xi_reach;      /* moment grid reach in sigma_xi = 2 sigma (24) */
    int window;           /* box window _window_pd (sgl_full.py:83-94, 254-258): 0 off (gauss
                             default), 1 always, 2 "auto" = only when |Phi| > phi_tol at a box
                             edge (the vp closure's default, pipeline.py:227-231) */
} sgl_invert_opts;

/* Grid and moments of one inversion (the reference's meta["grid"] and meta moments,
 * sgl_full.py:366-374). */
typedef struct {
    int64_t nk_k, nk_g, n_kap, n_gam;
    double k_k_max, k_g_max, kap_min, kap_max, gam_max, xi_min, xi_max, sigma;
    double phi_at_k_cut, phi_at_g_cut;
    double mean, var, skew, sigmaDL, norm;
    double ms_lambda, ms_transform, ms_path;   /* device time of the three stages */
    double window;                             /* 1 if the box window was applied */
    double xi_coarse, xi_coarse_k;             /* vp closure's coarse grid (gamma, kappa); 0 otherwise */
} sgl_invert_meta;

/* The inversion grid of one population (the reference's meta["grid"], sgl_full.py:187-262):
 * k_kappa = linspace(0, k_k_max, nk_k), k_gamma = linspace(0, k_g_max, nk_g); the output box
 * kappa = linspace(kap_min, kap_max, n_kap), gamma = linspace(0, gam_max, n_gam); sigma_kappa; and
 * |Phi| at the two reach cuts (they decide the "auto" window). */
typedef struct {
    int64_t nk_k, nk_g, n_kap, n_gam;
    double k_k_max, k_g_max, kap_min, kap_max, gam_max, sigma;
    double phi_at_k_cut, phi_at_g_cut;
} sgl_grid;

/* Library / context ------------------------------------------------------------------- */
int sgl_abi_version(void);

/* Creates a context on CUDA device `device` (its own stream, device arena). */
sgl_status sgl_ctx_create(int device, sgl_ctx** out);
void sgl_ctx_destroy(sgl_ctx* ctx);

/* Last error message of this context (or of the last failed sgl_ctx_create when ctx is
 * NULL), copied into buf.  Returns the message length. */
int sgl_last_error(const sgl_ctx* ctx, char* buf, int buflen);

/* The context's CUDA stream (a cudaStream_t), so a caller can record events on it. */
sgl_status sgl_ctx_stream(sgl_ctx* ctx, void** stream);

/* Per-kernel device-time statistics.  enable = 1 records CUDA events around every launch of
 * the engine's hot kernels (sweep, GEMMs, transforms, path integral) and accumulates, per kernel
 * tag: launches, device milliseconds, algorithmic FLOPs and bytes.  sgl_stats_json writes them
 * as a JSON object into buf (returns the full length); reset = 1 clears them afterwards.
 * No counterpart in the reference (its stage timers are wall-clock, pipeline.py:170-243). */
sgl_status sgl_ctx_profile(sgl_ctx* ctx, int enable);
int sgl_stats_json(sgl_ctx* ctx, char* buf, int buflen, int reset);

/* Population ---------------------------------------------------------------------------- */
/* Occupied fine (kappa, gamma) cells: weight w0, weight-averaged centroid (k0, g0), fine gamma
 * bin index ig, the fine gamma bin edges fe_g, and the weak-arm variance V.
 * Replaces the cell compaction of Lam.__init__ (sgl_full.py:2759-2775). */
sgl_status sgl_lam_set_cells(sgl_ctx* ctx, int64_t n_cells, const double* w0, const double* k0,
                             const double* g0, const int32_t* ig, const double* fe_g, int n_fe_g,
                             double V);

/* xi_lin two-point groups in the reference's raw form (Cells.xi_groups, sgl_full.py:1478-1523):
 * group g has harmonic m[g], nrow[g] rows over nidx[g] coarse cells (flat index idx into the
 * coarse lattice, gamma-fastest) plus one residual column: rows are nrow x (nidx + 1), row-major,
 * concatenated over groups.  ce_k / ce_g: coarse lattice edges.  prune: Lam's xi_prune (1e-7);
 * s0 > 0 overrides the largest row norm that prune is relative to (for subsets of groups).
 * Replaces the xi part of Lam.__init__ (sgl_full.py:2799-2861). */
sgl_status sgl_lam_set_xi(sgl_ctx* ctx, int n_groups, const int32_t* m, const int32_t* nrow,
                          const int32_t* nidx, const int32_t* idx, const double* rows,
                          const double* ce_k, int n_ce_k, const double* ce_g, int n_ce_g,
                          double prune, double s0);

/* Total sigma_kappa.  Replaces Lam.sigma (sgl_full.py:3437-3452) for the default chain. */
sgl_status sgl_lam_sigma(sgl_ctx* ctx, double* sigma);

/* ln Phi on the tensor grid kk x kg (row-major, nkk x nkg), real and imaginary planes.
 * Replaces Lam.__call__ / Lam._direct_call (sgl_full.py:3088-3160): the separable Psi_1 for
 * grids of >= 200000 points (direct sums otherwise), -1/2 k^2 V, and the gauss xi_lin term
 * (101^2 coarse grid + not-a-knot bicubic spline above 101^2 points, exact otherwise). */
sgl_status sgl_lnphi(sgl_ctx* ctx, const double* kk, int nkk, const double* kg, int nkg,
                     int precision, double* out_re, double* out_im);

/* The exact xi_lin (gauss) two-point term Psi_2 on the tensor grid kk x kg, without coarse-grid
 * interpolation, real and imaginary planes (nkk x nkg, row-major).  k_gamma = {0} and
 * k_kappa = {0} take the 1-D reach paths.  Replaces Lam._Qxi / Lam._Qxi_gauss
 * (sgl_full.py:2863-2951).  Requires sgl_lam_set_xi with at least one group. */
sgl_status sgl_xi_term(sgl_ctx* ctx, const double* kk, int nkk, const double* kg, int nkg, int precision,
                       double* out_re, double* out_im);

/* Positive (vp) Cox closure ---------------------------------------------------------------
 * Replaces the gauss xi_lin term by  q_xi = unwrap(ln R) - shear_var k_gamma^2 / 4  with
 *     ln R(k, q) = ln E_U exp( sum_s sum_g (lam_g(U_s) - 1) Y_g(k, q) ),
 *     Y_g = sum_{c in g} w_c (e_c J_c + J_c - 1),  e_c = expm1(i k kap_c),  J_c = J0(q gam_c)
 * over a stationary chain of nstate = 48 latent states (Closure.qxi pos_closure.py:690-705,
 * FusedVP.lnR_blocked pos_closure_fused.py:119-140, _chain_recursion pos_closure.py:184-240).
 * Arguments are the closure the reference's pos_closure.install (pos_closure.py:708-733) builds:
 * state nodes u and stationary weights w; n_shells - 1 transition matrices K[s][i][j] (row-major);
 * n_unique cells (ku, gu); n_cells group members (cu index into the unique cells, weight cw);
 * n_groups groups (members gstart[g] .. gstart[g+1]-1) in shells sh_g[s] .. sh_g[s+1]-1, each with
 * FusedVP's rate interval lam_g(u_j) - 1 = c + a (u_j - anchor) + b on states lo..hi (c = 0: all
 * states, anchor 0; c = -1: an interval reaching one end, anchor u_lo if hi = nstate-1, else u_hi;
 * rate_intervals pos_closure_fused.py:18-48).  Once set, sgl_lnphi / sgl_xi_term / sgl_pdf use it
 * (Lam._Qxi routed to the closure), sgl_pdf grows the coarse grid per axis with the box
 * (sgl_full.py:226-238), and sigma keeps the gauss groups' variance (Lam.sigma).
 * n_shells = 0 removes the closure. */
sgl_status sgl_vp_set(sgl_ctx* ctx, int nstate, const double* u, const double* w, int n_shells, const double* K,
                      int n_unique, const double* ku, const double* gu, int64_t n_cells, const int32_t* cu,
                      const double* cw, int n_groups, const int64_t* gstart, const int32_t* sh_g, const double* ga,
                      const double* gb, const double* gc, const int32_t* glo, const int32_t* ghi, double shear_var);

/* The same closure built by the engine from its per-shell population (the output of
 * pos_closure.population, pos_closure.py:388-450): cells of shell s at [shell_start[s],
 * shell_start[s+1]) with weight W, centroid (kap, gam) and loading phi; rho[s] the line-of-sight
 * correlation of shells s and s + 1 (n_shells - 1 values); fvar[s]; the kappa and gamma clustering
 * variance targets.  Builds nstate Gauss-Hermite latent states with stationary transitions, groups
 * each shell's cells by loading, calibrates eta (the model's kappa variance = target_kappa; eta_in
 * > 0 skips the calibration and uses it), forms the variance-preserving rates and their state
 * intervals and the unique cells, then installs the closure as sgl_vp_set does.  Replaces
 * Closure.__init__ / calibrate (pos_closure.py:453-591) and FusedVP's rate intervals
 * (pos_closure_fused.py:18-67).  *eta_out (may be NULL) receives eta. */
sgl_status sgl_vp_build(sgl_ctx* ctx, int nstate, int n_shells, const int64_t* shell_start, const double* W,
                        const double* kap, const double* gam, const double* phi, const double* rho,
                        const double* fvar, double target_kappa, double target_gamma, double eta_in,
                        double* eta_out);

/* ln R on the tensor grid kv x qv (nk x nq, row-major), principal branch, no shear term:
 * FusedVP.lnR_blocked (pos_closure_fused.py:119-140). */
sgl_status sgl_vp_lnR(sgl_ctx* ctx, const double* kv, int nk, const double* qv, int nq, int precision,
                      double* out_re, double* out_im);

/* One-dimensional compensated CF sweep over an arbitrary cell list (the synthetic plane x mass x
 * impact-parameter microbenchmark, 16.8M cells x 16384 k):
 *     out[n] = sum_c w_c (e^{i kk_n kap_c} - 1 - i kk_n kap_c)
 * the kappa part of the separable Psi_1 (A1 of _sep_lam_kernel, sgl_full.py:2596-2617).
 * set_cells uploads the cells once (host pointers); eval runs on a k grid (host in/out). */
sgl_status sgl_sweep_set_cells(sgl_ctx* ctx, int64_t n_cells, const double* kap, const double* w);
sgl_status sgl_sweep_eval(sgl_ctx* ctx, const double* kk, int nk, int precision, double* out_re,
                          double* out_im);

/* Surrogate MLP building blocks --------------------------------------------------------------
 * No counterpart in the reference: the learned per-plane log-CF model of the BF16 surrogate.
 * Device pointers; every call is asynchronous on the context's stream except sgl_mlp_mse.
 * sgl_gemm_bf16: C(i,j) = alpha sum_k A(i,k) B(k,j) with A(i,k) = A[i*a_rs + k*a_cs],
 *   B(k,j) = B[k*b_rs + j*b_cs], C(i,j) = C[i*c_rs + j*c_cs]; operands rounded to BF16 and packed for
 *   the tensor cores (tcgen05.mma.kind::f16, FP32 accumulation in TMEM).
 * sgl_mlp_bias_act: Zb = Z + bias[col], A = silu(Zb) (silu = 1) or Zb (silu = 0); M x N row-major.
 * sgl_mlp_act_grad: dZ = dA * silu'(Zb).   sgl_mlp_col_sum: out[j] = sum_i X[i, j] (FP64 sums).
 * sgl_mlp_mse: dpred = 2 (pred - target) / n and *loss = mean (pred - target)^2 (host, synchronous).
 * sgl_mlp_adamw: AdamW step `step` (>= 1) with bias-corrected moments, decoupled weight decay. */
sgl_status sgl_gemm_bf16(sgl_ctx* ctx, int M, int N, int K, const float* A, int64_t a_rs, int64_t a_cs,
                         const float* B, int64_t b_rs, int64_t b_cs, float* C, int64_t c_rs, int64_t c_cs,
                         float alpha);
sgl_status sgl_mlp_bias_act(sgl_ctx* ctx, int M, int N, const float* Z, const float* bias, float* Zb,
                            float* A, int silu);
sgl_status sgl_mlp_act_grad(sgl_ctx* ctx, int M, int N, const float* dA, const float* Zb, float* dZ);
sgl_status sgl_mlp_col_sum(sgl_ctx* ctx, int M, int N, const float* X, float* out);
sgl_status sgl_mlp_mse(sgl_ctx* ctx, int64_t n, const float* pred, const float* target, float* dpred,
                       double* loss);
/* sgl_mlp_infer: the trained 8 -> 6 x 256 SiLU -> 2 network's forward pass in one fused persistent kernel
 * (activations kept on chip as BF16 hi / lo parts, weights streamed by bulk copies, accumulation in TMEM):
 * X (n x 8) -> Y (n x 2), device float32; W, b: host arrays of the 7 layers' device pointers (W[l] in x out
 * row-major FP32 masters, rounded to BF16 as the training forward's GEMMs use them; b[l] FP32).  The
 * arithmetic is the training forward's (split BF16 inputs, BF16 weights, FP32 accumulation). */
sgl_status sgl_mlp_infer(sgl_ctx* ctx, int n, const float* X, int n_layers, const float* const* W, const float* const* b,
                         float* Y);
sgl_status sgl_mlp_adamw(sgl_ctx* ctx, int64_t n, float* w, const float* g, float* m, float* v, float lr,
                         float b1, float b2, float eps, float wd, int step);

/* Measured FMA throughput of this GPU (fp64 = 1: FP64, 0: FP32), TFLOP/s (2 flops per FMA):
 * the denominator of the CF-sweep roofline.  No counterpart in the reference. */
sgl_status sgl_measure_peak(sgl_ctx* ctx, int fp64, double* tflops);

/* Fills opts with the pipeline defaults above. */
void sgl_invert_opts_default(sgl_invert_opts* opts);

/* Phi = exp(ln Phi) -> P_s(ln mu) at xi_out (n_xi points), normalised on the wide grid.
 * Replaces sgl_full.invert (sgl_full.py:159-375) with sgl.vector_grid (sgl.py:1229-1258) and
 * sgl.P_vector_joint (sgl.py:1127-1156): measured k-reach, width-relative grid with the tail
 * box, Hankel + Fourier transforms, Euler-Maclaurin endpoint term, constant-mu path integral.
 * Grids above 2e7 k-points, which the reference inverts in k_kappa row blocks (_invert_blocked,
 * sgl_full.py:97-157), run the same sums unblocked in device memory (up to 65535 k_kappa rows);
 * SGL_ERR_CUDA reports an allocation that does not fit.  P_out: n_xi doubles (host).  meta may
 * be NULL. */
sgl_status sgl_pdf(sgl_ctx* ctx, const double* xi_out, int n_xi, const sgl_invert_opts* opts,
                   double* P_out, sgl_invert_meta* meta);

/* The grid half of sgl_pdf: vector_grid (sgl.py:1229-1258), the tail box and the measured k-reach
 * (_reach, sgl_full.py:38-47; the grid logic of invert, sgl_full.py:187-262) for the context's
 * population, without evaluating Phi on the grid.  With the vp closure installed its coarse grid
 * grows with the box, as in sgl_pdf. */
sgl_status sgl_plan_grid(sgl_ctx* ctx, const sgl_invert_opts* opts, sgl_grid* grid);

/* The inversion half of sgl_pdf for a caller-owned Phi: Phi = exp(ln Phi) on the grid's tensor k
 * grid as two FP64 planes (re, im; nk_k x nk_g row-major), host pointers (phi_on_device = 0) or
 * device pointers on the context's device (1).  Applies the window (opts->window), the Hankel and
 * kappa transforms with the Euler-Maclaurin term, the constant-mu path integrals, normalisation and
 * moments: the part of sgl_full.invert after `Phi = np.exp(lam(k_k, k_g))` (sgl_full.py:272-375,
 * sgl.P_vector_joint sgl.py:1127-1156).  For SGL_MIXED Phi is rounded to FP32 first.  Given the grid
 * sgl_plan_grid returns and exp(sgl_lnphi) on it, the result is sgl_pdf's.  Needs no population. */
sgl_status sgl_invert(sgl_ctx* ctx, const double* phi_re, const double* phi_im, int phi_on_device,
                      const sgl_grid* grid, const double* xi_out, int n_xi, const sgl_invert_opts* opts,
                      double* P_out, sgl_invert_meta* meta);

/* Batched plain solver -----------------------------------------------------------------------
 * No counterpart in the reference, which solves one pipeline.run per PDF (pipeline.py:114-274).
 * A batch owns `slots` contexts on one device; load each slot's population through the context
 * sgl_batch_slot returns (sgl_lam_set_cells / sgl_lam_set_xi / sgl_vp_set), then sgl_batch_pdf runs
 * n_jobs PDFs, job j on slot job_slot[j] (a slot may take many jobs; they run in order), all with
 * the same options and ln mu grid: P_out is n_jobs x n_xi, meta (optional) n_jobs entries,
 * job_status (optional) each job's status (SGL_ERR_STATE: not run because an earlier job of its
 * slot failed).  The slots run concurrently, each on its own host thread of the batch and its own
 * streams.  Returns the first failure (message: sgl_last_error(NULL, ...)).  The slot contexts
 * belong to the batch: do not destroy them. */
typedef struct sgl_batch sgl_batch;
sgl_status sgl_batch_create(int device, int slots, sgl_batch** out);
void sgl_batch_destroy(sgl_batch* batch);
int sgl_batch_slots(const sgl_batch* batch);
sgl_ctx* sgl_batch_slot(sgl_batch* batch, int slot);
sgl_status sgl_batch_pdf(sgl_batch* batch, int n_jobs, const int32_t* job_slot, const double* xi_out, int n_xi,
                         const sgl_invert_opts* opts, double* P_out, sgl_invert_meta* meta, int32_t* job_status);

/* Batched CF solver over uneven instances ------------------------------------------------------
 * No counterpart in the reference (one pipeline.run per instance, pipeline.py:114-274).  Instance i
 * has planes inst_plane0[i] .. inst_plane0[i+1]-1; plane p has cells plane_cells[p] ..
 * plane_cells[p+1]-1 (kap, w); its k grid is k_n = n dk[i], n < nk[i].  Its log-CF:
 *   closure[i] = 0 (gauss): sum_c w (e^{i k kap} - 1 - i k kap) - V[i] k^2 / 2
 *   closure[i] = 1 (vp):    sum_p Lambda_p(k) + ln E exp(sum_p (lam_p(U_p) - 1) Lambda_p(k)), U a stationary
 *                           chain on nstate (<= 8) states: vp_D[p][s] = lam_p(u_s) - 1 per plane, and per vp
 *                           instance (in order) vp_K[s][t] (transition) and vp_w[s] (stationary weights) --
 *                           the positive Cox closure's chain (pos_closure.py:184-240) with one group per plane.
 * sgl_cfb_set uploads the batch (host arrays).  sgl_cfb_tune times every (k points per work item, CTAs per
 * SM) shape on a work-bounded sample of the batch and keeps the fastest (SGL_MIXED; SGL_FP64 takes 128
 * k-points per item and every resident CTA); it runs on first use otherwise, once per batch shape class
 * (largest k grid and mean cells per instance, in powers of two) and context.
 * sgl_cfb_lnphi runs the persistent solve (one launch; CTAs take (instance, k tile) items from a device
 * counter, longest instances first) and copies ln Phi out as (re, im) pairs per k, instances in order
 * (out may be NULL).  sgl_cfb_pdf adds Phi = exp(ln Phi) and the inversion to dP/dln mu at the n_lnmu
 * points (mu = (1 - kappa)^-2): P_out is n_inst x n_lnmu; use_graph = 1 captures the whole step in a CUDA
 * graph on first use and replays it; *ms_out (may be NULL) receives the device time of the step. */
sgl_status sgl_cfb_set(sgl_ctx* ctx, int n_inst, const int32_t* inst_plane0, const int64_t* plane_cells,
                       const double* kap, const double* w, const int32_t* nk, const double* dk, const int32_t* closure,
                       const double* V, int nstate, const double* vp_D, const double* vp_K, const double* vp_w);
/* sgl_cfb_set_separable: a gauss-closure batch whose planes share one nm x nb cell template, built on the
 * device: cell (m, b) of plane p (planes in order, nm * nb cells each) has kap = u[p][m] F[m][b] and
 * w = v[p][m] g[b] (F nm x nb row-major, g nb, u and v n_planes x nm; host arrays).  k0 (may be NULL =
 * zeros) offsets instance i's k points to k0[i] + n dk[i] for sgl_cfb_lnphi, or with geom = 1 makes them
 * log-spaced, exp(k0[i] + n dk[i]) (sgl_cfb_pdf needs k0 = 0 and geom = 0).  A new batch keeps the launch
 * shapes tuned for the previous one. */
sgl_status sgl_cfb_set_separable(sgl_ctx* ctx, int nm, int nb, const double* F, const double* g, int n_inst,
                                 const int32_t* inst_plane0, const int32_t* nk, const double* dk, const double* k0,
                                 int geom, const double* V, const double* u, const double* v);
sgl_status sgl_cfb_tune(sgl_ctx* ctx, int precision, int* kt, int* ctas_per_sm);
sgl_status sgl_cfb_lnphi(sgl_ctx* ctx, int precision, double* out);
sgl_status sgl_cfb_pdf(sgl_ctx* ctx, int precision, const double* lnmu, int n_lnmu, double* P_out, int use_graph,
                       double* ms_out);

/* Surrogate + judge production sweep ------------------------------------------------------------
 * No counterpart in the reference.  Instances i < n_inst with planes inst_plane0[i] .. inst_plane0[i+1]-1
 * and uniform k grids k_n = n dk[i], n < nk[i]; plane p adds dz[p] H_p(s[p] k) to its instance's log-CF.
 * H_p comes from a surrogate ensemble at nq >= 4 nodes ln q_j = lnq0[p] + j hq[p] as the residual over the
 * plane's two-moment form H0(q) = -(mu2 / 2) q^2 / (1 - i q Sbar), Sbar = mu2 / (2 mu1) (mu1, mu2 > 0: the
 * plane's sum w S and sum w S^2):  ln |H| = r0 + ln |H0|,  arg(-H) = r1 + arg(-H0)  (host arrays, sgl_sur_set).
 * Y (device, float32) holds the members' normalised outputs [member][plane][node] = (y0, y1), r0 = y0 scale
 * + shift, r1 = y1 scale; between nodes 4-point Lagrange interpolation, below the first node r q / q0.
 * sgl_sur_judge sums the ensemble mean into ln Phi per instance and returns per plane dis_out (2 floats:
 * the largest dz |spread| over the k grid, as is and weighted by |Phi| of the surrogate sum; spread =
 * 2 max_m |H_m - mean|) and band_out (2 ints: the first k index whose weighted spread exceeds tau and 1 +
 * the last; 0, 0 if none).  sgl_sur_finish recomputes ln Phi with plane p taken, on k_n for exact_lo[p] <= n
 * < exact_lo[p] + nk', from instance exact_inst[p] of the batched solver's last sgl_cfb_lnphi (its nk', dk
 * equal, k0 = exact_lo[p] dk; exact_inst -1 = surrogate only; exact_lo may be NULL = zeros).  sgl_sur_pdf
 * inverts the current ln Phi to dP/dln mu at n_lnmu points (as sgl_cfb_pdf; P_out n_inst x n_lnmu) and
 * copies ln Phi out as (re, im) pairs when lnphi_out is not NULL. */
sgl_status sgl_sur_set(sgl_ctx* ctx, int n_inst, const int32_t* inst_plane0, const int32_t* nk, const double* dk,
                       const double* s, const double* dz, const double* mu1, const double* mu2, const double* lnq0,
                       const double* hq, int nq);
sgl_status sgl_sur_judge(sgl_ctx* ctx, const float* Y, int members, double shift, double scale, double tau,
                         float* dis_out, int32_t* band_out);
sgl_status sgl_sur_finish(sgl_ctx* ctx, const float* Y, int members, double shift, double scale,
                          const int32_t* exact_inst, const int32_t* exact_lo);
sgl_status sgl_sur_pdf(sgl_ctx* ctx, int precision, const double* lnmu, int n_lnmu, double* P_out, double* lnphi_out);
/* sgl_sur_nodes_exact: instance j of the batched solver's last sgl_cfb_lnphi holds plane planes[j]'s cells
 * on the k points of its nodes node_lo[j] .. node_lo[j] + nk_j - 1 (log-spaced: sgl_cfb_set_separable with
 * geom = 1, k0 = lnq0 - ln s + node_lo hq, dk = hq; node_lo may be NULL = zeros), so its ln Phi is
 * dz H(q_node); writes those nodes' normalised residuals into every member's slots of Y (device), which the
 * next sgl_sur_judge / sgl_sur_finish then interpolate. */
sgl_status sgl_sur_nodes_exact(sgl_ctx* ctx, int n, const int32_t* planes, const int32_t* node_lo, float* Y,
                               int members, double shift, double scale);

/* Cosmology tables ------------------------------------------------------------------------------------
 * Replaces the chain's Cosmology (sgl.py:65-640 as pipeline.make_cosmology builds it, pipeline.py:39-79:
 * EH98 transfer, smooth-k sigma(M) window with the top-hat sigma_8 anchor, Ludlow+16 concentrations, the
 * growth ODE, radiation Omega_r = Om / (1 + z_eq)) for n cosmologies at once, one CTA each.  params: n x 9
 * (h, Om, Ob, s8, ns, zeq, Ok, w0, wa), checked against the reference's domain (SGL_ERR_VALUE).  At the nz
 * ascending redshifts z: E, chi (radial comoving distance, Mpc), DM (transverse), D (growth, D(0) = 1), each
 * n x nz; at the nm masses M (Msun): sigmaM (sigma(M) at z = 0) and dlnsig (d ln sigma / d ln M), n x nm; at
 * the nzm redshifts zm: dndlnM (Sheth-Tormen, Mpc^-3) and conc (c_200c), n x nzm x nm.  All host arrays. */
sgl_status sgl_cosmo_tables(sgl_ctx* ctx, int n, const double* params, int nz, const double* z, int nm, const double* M,
                            int nzm, const double* zm, double* E, double* chi, double* DM, double* D, double* sigmaM,
                            double* dlnsig, double* dndlnM, double* conc);

/* Binned-cell deposit of the population build ------------------------------------------------------------
 * Replaces the build's Cells accumulator (sgl_full.py:1282-1533): every emitter's points binned on the fine
 * and coarse (kappa, gamma) lattices, which stay in device memory between calls.
 * sgl_cells_init starts a build (the context holds one): nshell shells, moments n = 0..nord, the lattices'
 * edges (ascending; kappa signed-log, gamma geometric, as Cells.fe / Cells.ce, sgl_full.py:1293-1294; at most
 * 6144 edges in all), gamma clipped below at g_clip (sgl_full.py:1324: 1.0000001 x the fine grid's lowest
 * gamma), and k_max_fine, the |kappa| bound of the linear sums (the fine grid's top kappa).
 * sgl_cells_add deposits n_obj objects in order (Cells.add, sgl_full.py:1314-1385): object o is points
 * off[o] .. off[o + 1] - 1 of K, G, W (and R), in shell[o] with bias weight beta[o] (finite) and tangential
 * shear tang[o] (NULL = all tangential).  Bins are searchsorted(side='right') with the last edge in the last
 * bin, exactly; a point adds w, w kappa, w gamma to its fine bin and w beta^n to its coarse bin of its shell.
 * sums (n_obj x 3, host) receives each object's total w, w inside the fine lattice, and w kappa over
 * |kappa| < k_max_fine, from which the caller keeps N, dropped and lin.  Bin sums are FP64 atomics: the
 * reference's sums in another order.  All point arrays are host arrays.
 * sgl_cells_xi_init turns on the xi_lin term (Cells(xi=...), sgl_full.py:2483-2512): nkp <= 64 k_perp nodes
 * kp with weights c, mmax <= 2, pos = 1 for the positive closure's rate deposit; every deposit then needs R
 * (the lens distance of each point, Mpc) inside a node opened by sgl_cells_xi_begin (dchi, Mpc) and closed by
 * sgl_cells_xi_end (sgl_full.py:1478-1523), which compresses the node into *n_groups row groups fetched by
 * sgl_cells_xi_group (m, nidx, nrow; then idx nidx ints, rows nrow x (nidx + 1), for m = 0 with pos also W
 * nidx and v0 nkp; any output may be NULL).  Rows are fixed up to sign and rotation within the kept modes.
 * sgl_cells_xi_shear_tail adds the analytic shear tail beyond radius Rm (sgl_full.py:1466-1476).
 * sgl_cells_read copies the lattices out: H0, H0k, H0g (fine, nkf x ngf) and Hc (nshell x (nord+1) x nkc x
 * ngc); any may be NULL. */
sgl_status sgl_cells_init(sgl_ctx* ctx, int nshell, int nord, int nekf, const double* ekf, int negf,
                          const double* egf, int nekc, const double* ekc, int negc, const double* egc,
                          double g_clip, double k_max_fine);
sgl_status sgl_cells_add(sgl_ctx* ctx, int n_obj, const int64_t* off, const double* K, const double* G,
                         const double* W, const double* R, const int32_t* shell, const double* beta,
                         const unsigned char* tang, double* sums);
sgl_status sgl_cells_xi_init(sgl_ctx* ctx, int nkp, const double* kp, const double* c, int mmax, int pos);
sgl_status sgl_cells_xi_begin(sgl_ctx* ctx, double dchi);
sgl_status sgl_cells_xi_shear_tail(sgl_ctx* ctx, double beta, double Gam, double Rm, double n_area);
sgl_status sgl_cells_xi_end(sgl_ctx* ctx, int* n_groups);
sgl_status sgl_cells_xi_group(sgl_ctx* ctx, int g, int32_t* m, int32_t* nidx, int32_t* nrow, int32_t* idx,
                              double* rows, double* W, double* v0);
sgl_status sgl_cells_read(sgl_ctx* ctx, double* H0, double* H0k, double* H0g, double* Hc);

/* Allocation-free entry point ------------------------------------------------------------
 * No counterpart in the reference.  For callers that may not allocate device memory (a host that
 * gives its whole device budget to its own pool or caching allocator, or that forbids third-party
 * allocations on its streams): computes the kappa-axis Poisson exponent
 *     out[n] = sum_c w0_c (e^{i kk_n k0_c} - 1 - i kk_n k0_c)      (FP64; = sgl_lnphi at k_gamma = 0
 *                                                                   for cells with V = 0 and no xi)
 * with no cudaMalloc / cudaFree and no context.  Partial sums live in one fixed 8 MiB file-scope
 * device array (16 x 32768 double2) that every GPU loading the library holds until exit; nk is
 * limited to 32768 and larger nk is rejected (SGL_ERR_VALUE).  kk, k0, w0, out_re, out_im are
 * device-accessible pointers; stream is a cudaStream_t (NULL = legacy default stream); the call
 * is asynchronous on that stream.  Every call looks up the array's device address
 * (cudaGetSymbolAddress) with the caller's device current; the first call on a device may load
 * the library's device code there, so make it before any stream capture.
 * All calls share the array, so calls that overlap on the GPU (other streams, other threads)
 * race; every partial the call reads is written by the same call, so nothing needs clearing.
 * Errors: sgl_last_error(NULL, ...). */
sgl_status sgl_cf_kappa_noalloc(const double* kk, int nk, const double* k0, const double* w0,
                                int64_t n_cells, double* out_re, double* out_im, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* SGL_GB300_H */
