// Internal launcher declarations shared by the .cu translation units.
#pragma once
#include "common.cuh"
#include "gemm.cuh"

namespace sgl {

// Separable Psi_1 plan on the device (cells sorted by gamma-node group).
struct SepDevice {
    int n_cells = 0, n_groups = 0, n_cols = 0, n_cols_sep = 0, nchunks = 0;
    const double* kap = nullptr;      // [n_cells] centroid kappa
    const double* w = nullptr;        // [n_cells] weight
    const double* wl = nullptr;       // [n_cells * 8] weight x Lagrange basis (direct cells: w, 0...)
    const float* kap_hi = nullptr;    // float-float kappa (mixed path)
    const float* kap_lo = nullptr;
    const float* w_f = nullptr;
    const float* wl_f = nullptr;
    const int* grp = nullptr;         // [n_cells] group of each cell
    const int* gcol0 = nullptr;       // [n_groups] first T column
    const int* gncol = nullptr;       // [n_groups] 8 (Chebyshev nodes) or 1 (exact node)
    const int* chunk_begin = nullptr; // [nchunks + 1] cell offsets (group aligned)
};

// ---- Psi_1
int psi1_direct_chunks(int64_t nc);
void launch_psi1_direct(const double* kk, int nk, const double* kg, int nkg, const double* k0,
                        const double* g0, const double* w0, int64_t nc, double* re, double* im,
                        double2* part, cudaStream_t st, int precision = SGL_FP64);
void launch_sep_sweep(int precision, const double* kk, int nk, const SepDevice& s, void* Tt,
                      double2* A_part, double2* A1, cudaStream_t st);
void launch_j0m1_table(int precision, const double* nodes, int nn, const double* x, int nx, void* B,
                       cudaStream_t st);
void launch_cheb_matrix(int precision, double K, int N, const double* tpts, const double* x, int nx, void* L,
                        cudaStream_t st);
void launch_cheb_points(double K, int N, double* t, cudaStream_t st);

// ---- GEMM
constexpr int kSmallTiles = 100;   // launch_grouped_gemm layout code for 16 x 16 FP64 tiles
template <typename T>
void launch_grouped_gemm(const GemmDesc<T>* d_descs, int nprob, int tiles, int layout, cudaStream_t st);
template <typename T>
void launch_sum_slices(const T* ws, int nslices, int rows, int cols, T* out, long long ldo, T beta, cudaStream_t st);

// ---- xi_lin (gauss) Psi_2
struct XiDevice {
    int n_groups = 0, n_kmc = 0, n_gmc = 0;
    const double* kmc = nullptr;       // [n_kmc] coarse kappa centres
    const double* gmc = nullptr;       // [n_gmc] coarse gamma centres
    // per group
    const int* g_m = nullptr;
    const int* g_r = nullptr;
    const int* g_nP = nullptr;
    const long long* g_p_off = nullptr;     // into idx_p / p_ptr rows
    const long long* g_ent_off = nullptr;   // into ent_q / rows columns
    const long long* g_row_off = nullptr;   // into rows / res / sum_rows (row units)
    const int* idx_p = nullptr;        // global kappa-centre index of each local p
    const int* p_ptr = nullptr;        // CSR over local p: entries [p_ptr[p], p_ptr[p+1]) (group relative)
    const int* ent_qg = nullptr;       // global gamma-centre index of each entry
    const double* rows = nullptr;      // rows: entry-major per group: rows[(ent_off + e) * r + rr]
    const float* rows_f = nullptr;     // float copy of rows (mixed path)
    int r_max = 0;                     // largest group row count
    const int* g_nQ = nullptr;         // unique gamma cells per group
    const long long* g_q_off = nullptr;   // into idx_q
    const long long* g_u_off = nullptr;   // into U0 (r x nQ per group)
    const int* idx_q = nullptr;        // global gamma-centre index of each local q
    const double* U0 = nullptr;        // sum over p of the rows (m = 0 groups; zeros otherwise)
    const double* res = nullptr;       // [total rows]
    const double* sum_rows = nullptr;  // [total rows]
    // 1-D reach paths
    int R0 = 0;
    const double* W0 = nullptr;        // [R0 * n_kmc]
    const double* res0 = nullptr;
    const double* sum0 = nullptr;
    int Rm[3] = {0, 0, 0};
    const double* U[3] = {nullptr, nullptr, nullptr};    // [Rm * n_gmc]
    const double* resm[3] = {nullptr, nullptr, nullptr};
    const double* summ[3] = {nullptr, nullptr, nullptr};
};

void launch_xi_line_k(const XiDevice& x, const double* kk, int nk, double* out_re, double* out_im, double* part,
                      cudaStream_t st);
void launch_xi_line_g(const XiDevice& x, const double* kg, int nkg, double* out_re, double* out_im, double* part,
                      cudaStream_t st);
constexpr int kLineChunks = 32;   // row chunks of the 1-D reach paths (part: 3 * kLineChunks * points)
void launch_bessel_tables(int precision, const double* gmc, int n_gmc, const double* kg, int nkg, void* J, cudaStream_t st);
void launch_xi_stageA(int precision, const XiDevice& x, const long long* h_p_prefix, int total_p, const long long* T_off,
                      const void* J, int nkg, void* T, cudaStream_t st);
void launch_xi_E(int precision, const XiDevice& x, const double* kk, int nk, const long long* E_off,
                 const long long* h_p_prefix, int total_p, void* E, cudaStream_t st);
void launch_xi_square(int precision, const XiDevice& x, const long long* G_off, const void* G, const double* kk, int nk,
                      const double* kg, int nkg, const double* V, int nsplit, double* part, double* out_re,
                      double* out_im, cudaStream_t st);
void launch_xi_V(const XiDevice& x, const double* J0m1, int nkg, double* V, int total_rows, cudaStream_t st);
void launch_xi_V_mixed(const XiDevice& x, const double* J0m1, int nkg, float* Vf, int total_rows, const double* kk,
                       int nk, const double* kg, float2* kres, float2* hq, cudaStream_t st, int kres_t = 0);
// fused mixed gauss Psi_2 (tcgen05; xi_fused.cu): T built in shared memory, contracted with the
// packed E in TMEM, squared and summed over rows in the epilogue
int xi_fused_jt(int r);
constexpr int kXiTailPad = 16;     // elements after rows_f and ent_qg: room for 16-byte-aligned bulk copies
bool xi_fused_fits(int r_max, int nk, int n_gmc);
void launch_xi_E_pack(const XiDevice& x, const double* kk, int nk, const long long* pp_prefix, long long total_pp,
                      const long long* p_prefix, const long long* e_off, float* Epk, cudaStream_t st);
void launch_xi_fused(const XiDevice& x, const long long* p_prefix, const long long* rowel_off, const int* jt,
                     const long long* cta_prefix, long long ctas, const long long* e_off, const float* Epk,
                     const float* J, const float* Vf, const float2* kresT, const float2* hq, int nk, int nkg,
                     float2* part, int* err, double* out_re, double* out_im, cudaStream_t st);
void launch_xi_square_mixed(const XiDevice& x, const long long* G_off, const float* G, int nk, int nkg, const float* Vf,
                            const float2* kres, const float2* hq, int rows, int nsplit, double* part, double* out_re,
                            double* out_im, cudaStream_t st);

// ---- spline + composition
struct SplineAxis {              // per evaluation point: interval l (first coefficient) + 4 weights
    const int* l = nullptr;
    const double* b = nullptr;   // [n * 4]
    const float* bf = nullptr;   // FP32 copy of b (mixed path), or null
};
void launch_to_float(const double* src, float* dst, long long n, cudaStream_t st);
void launch_spline_basis(const double* x, int n, double xmax, const double* knots, int ncoef, int* l, double* b,
                         cudaStream_t st);
// out = G + A1[n] - 1/2 kk^2 V + spline(C) ; mode 0: write lnPhi (double planes), mode 1: write Phi (TT planes)
// Cf (mixed path, optional): FP32 copies of C_re then C_im (2 ncoef_k ncg floats) for an FP32 spline
// evaluation; sk.bf and sg.bf must then be set too.
void launch_finalize(int precision, int write_phi, const void* G, int nk, int nkg, const double2* A1, const double* kk,
                     double V, const double* C_re, const double* C_im, int ncg, SplineAxis sk, SplineAxis sg,
                     void* out_re, void* out_im, long long ld_out, cudaStream_t st, const float* Cf = nullptr,
                     long long nq = 0);

// ---- inversion
void launch_hankel_matrix(int precision, const double* kg, int nkg, double dkg, const double* gam, int ngam, int ld,
                          void* M, cudaStream_t st);
void launch_kappa_matrix(int precision, const double* kk, int nk, double dkk, const double* kap, int nkap, void* CS,
                         cudaStream_t st);
void launch_em_columns(int precision, const void* Phi, int nk, int nkg, double dkg, void* F, int ldF, int col,
                       cudaStream_t st);
void launch_window(int precision, void* Phi, int nk, int nkg, const double* wk, const double* wg, cudaStream_t st);
void launch_phi_to_f32(const double* in, long long n, float* out, cudaStream_t st);

// ---- batched CF solver (cfbatch.cu)
struct CfbInst {                          // one instance of the batch
    long long c0, c1;                     // its cells (all planes)
    long long k_off;                      // first k-point in the per-instance output arrays
    int p0, p1;                           // its planes
    int nk, closure;                      // k points (k_n = n dk); closure 0 gauss, 1 vp
    double dk, V;                         // k step; gauss: the clustering variance term V k^2 / 2
    int vp_slot;                          // vp: index into the chain tables
    int geom;                             // 1: the solve's k points are exp(k0 + n dk) (log-spaced)
    double k0;                            // else k0 + n dk (the inversion assumes k0 = 0)
};
void launch_cfb_persistent(int precision, int kt, int ctas, const CfbInst* inst, const int2* items, int n_items,
                           int* counter, const long long* plane_cells, const double* kap, const double* w,
                           const float* kh, const float* kl, const float* wf, const double* vp_D, const double* vp_K,
                           const double* vp_w, int nstate, double2* out, cudaStream_t st);
void launch_cfb_pdf(int precision, const CfbInst* inst, int n_inst, const double2* lnphi, long long total,
                    const long long* k_offs, void* phi, const double* lnmu, int nm, double* P, cudaStream_t st);
int cfb_resident_ctas(int precision, int kt);
void launch_cfb_fill_separable(long long n_cells, int nm, int nb, const double* F, const double* g, const double* u,
                               const double* v, double* kap, double* w, float* kh, float* kl, float* wf, cudaStream_t st);
struct SurPlane {                         // one plane of the surrogate sweep
    double s, dz;                         // lensing efficiency, thickness: the plane adds dz H(s k)
    double lnq0, hq;                      // its surrogate nodes ln q_j = lnq0 + j hq
    double lnmu2h, sbar;                  // two-moment form: ln(mu2 / 2), Sbar = mu2 / (2 mu1)
    long long exact_off;                  // finishing pass: first k of its exact ln Phi, or -1
    int exact_lo, exact_nk;               // exact for k_n, exact_lo <= n < exact_lo + exact_nk
};
void launch_sur_nodes_exact(int n, const int* planes, const int* node_lo, const CfbInst* cfb_inst,
                            const double2* cfb_lnphi, const SurPlane* sp, int nq, float* Y, long long y_member_stride,
                            int members, float shift, float scale, cudaStream_t st);
void launch_sur_sum(bool judge, const CfbInst* inst, int n_inst, int max_nk, const SurPlane* planes, const float* Y,
                    long long y_member_stride, int members, int nq, float shift, float scale, float tau,
                    const double2* exact, double2* lnphi, unsigned int* dis, int* first, int* last, cudaStream_t st);
long long cosmo_work_doubles(int nx);
void launch_cosmo_tables(int n, const double* params, int nz, const double* z, const double* x_out, const int* x_slot,
                         int nx, int nm, const double* M, int nzm, const double* zm, double A_st, double* E,
                         double* chi, double* DM, double* D, double* Dm, double* sigM, double* dlnsig,
                         double* dndlnM, double* conc, double* work, cudaStream_t st);
void launch_p3_finish(int precision, const void* P3ext, int nkap, int ngam, int ld, const double* gam, double* P3,
                      float* P3f, cudaStream_t st);
void launch_path_integral(const double* P3, const float* P3f, int nkap, int ngam, double kap0, double kap1,
                          double gam1, const double* xi, int nxi, double gmax, double g_def, int n_k_int, double* out,
                          cudaStream_t st);

// ---- tcgen05 grouped GEMM (TF32 hi/lo split, FP32 accumulation in TMEM)
struct TcGemmDesc {
    int M, N, K;
    const float* A; long long a_rs, a_cs;   // A(i,k) = A[i*a_rs + k*a_cs]
    const float* B; long long b_rs, b_cs;   // B(k,j) = B[k*b_rs + j*b_cs]
    float* C; long long c_rs, c_cs;         // C(i,j) = alpha * sum_k A(i,k) B(k,j) at C[i*c_rs + j*c_cs]
    float alpha;
    // filled by tc_gemm_plan
    int tile_begin, tiles_n, bn, Mpad, Npad;
    long long a_off, b_off;                 // packed operands (floats into the packed buffer)
};
struct TcPackDesc {                         // one operand to pack: X(r, k) = X[r*x_rs + k*x_cs]
    const float* X; long long x_rs, x_cs;
    int R, K, Rpad, nkb;
    long long out_off, quad_begin;
};
// fills tiles / packing descriptors (pk: 2 n entries) for operands split into `parts` (2 or 3)
// TF32 parts; returns the packed buffer size in floats
long long tc_gemm_plan(TcGemmDesc* d, int n, int parts, TcPackDesc* pk, int* tiles, long long* quads,
                       bool pack_a = true, int bn_max = 256);
// FP32 GEMM with the TMEM accumulation drained every 64 products into TwoSum running sums (tiles of
// at most tc_drain_bn() columns: plan with bn_max = tc_drain_bn())
void launch_tc_gemm_drain(int parts, const TcGemmDesc* d_descs, int nprob, int tiles, const TcPackDesc* d_pack,
                          long long quads, float* packed, int* err, cudaStream_t st);
int tc_drain_bn();
void launch_tc_gemm(int parts, const TcGemmDesc* d_descs, int nprob, int tiles, const TcPackDesc* d_pack,
                    long long quads, float* packed, int* err, cudaStream_t st);

// gauss stage A of the mixed path written as the packed (2-part TF32) A operand of the xi GEMM
bool xi_stageA_pack_fits(int r_max, int nkg);
void launch_xi_stageA_pack(const XiDevice& x, const long long* d_p_prefix, const float* J, int nkg,
                           const long long* d_chunk_prefix, long long nchunks, const TcGemmDesc* d_descs,
                           float* packed, cudaStream_t st);

// ---- surrogate MLP element-wise kernels
int mlp_fused_smem();
int mlp_fused_small_floats();
long long mlp_fused_wp_bytes();
sgl_status mlp_fused_attr();
void launch_mlp_fused(int n, const float* X, const float* const* W_dev, const float* const* b_dev, unsigned char* Wp,
                      float* small, const float** ptrs, float* Y, int* err, int ctas, cudaStream_t st);
void launch_bias_act(int M, int N, const float* Z, const float* bias, float* Zb, float* A, int silu, cudaStream_t st);
void launch_act_grad(int M, int N, const float* dA, const float* Zb, float* dZ, cudaStream_t st);
void launch_col_sum(int M, int N, const float* X, float* out, cudaStream_t st);
int mse_blocks(long long n);
void launch_mse(long long n, const float* pred, const float* tgt, float* dpred, double* part, cudaStream_t st);
void launch_adamw(long long n, float* w, const float* g, float* m, float* v, float lr, float b1, float b2, float eps,
                  float wd, float c1, float c2, cudaStream_t st);

// ---- device-side xi group preparation (coherent host-memory access)
struct XiPrepRow {                 // one kept row
    long long src;                 // first element of the raw row in the caller's rows
    long long dst;                 // rows_t offset of entry 0 of its group, + rr
    long long ent0;                // group's first entry (inverse / q / p orders)
    long long u_off, u0_off, w0_off;   // row starts in U[m], U0, W0
    int ne, R, row, m;             // entries, kept rows of the group, global kept-row index, harmonic
    int nQ, q0, qseg0;             // gamma cells: count, offset into idx_q, offset into qseg
    int nP, p0;                    // kappa cells: count, global p offset (p_ptr / idx_p)
};
struct XiPrepIdx {
    const int* qord;               // [entries] entries sorted by gamma cell (stable)
    const int* qseg;               // per group: nQ + 1 segment starts into qord
    const int* pord;               // [entries] entries in p-order
    const int* p_ptr;              // global CSR over p-ordered entries
    const int* idx_p;              // global kappa-cell index of each p
    const int* idx_q;              // global gamma-cell index of each q
};
struct XiPrepOut {
    double* rt; float* rtf; double* res; double* sums; double* sig;
    double* U; double* U0; double* W0;
};
void launch_xi_stage_rows(const double* rows, long long n, double* dst, cudaStream_t st);
// bytes must be a multiple of 4, both pointers 4-byte aligned; src is host memory the device
// reads coherently
void launch_copy_from_host(const void* src, size_t bytes, void* dst, cudaStream_t st);
void launch_xi_row_norms(const double* rows, const long long* row_start, const int* row_len, int nrows,
                         double* norms, cudaStream_t st);
// tiles: (first kept row of the group in kr, first entry i0); at most 256 kept rows per group
void launch_xi_transpose(const double* rows, const XiPrepRow* kr, const int2* tiles, int ntiles, const int* pord,
                         double* rt, float* rtf, cudaStream_t st);
void launch_xi_rowprep(const double* rows, const XiPrepRow* kr, int nkept, int ne_max, const XiPrepIdx& ix,
                       const double* kmc, const XiPrepOut& o, cudaStream_t st);

// ---- positive (vp) Cox closure
// Cells sorted per shell into runs (one kind and interval bound; runs ordered linear first, then by
// the first state they change: lo for left runs, hi + 1 for right runs), per-cell weights (w a, w b).
struct VpDevice {
    int nsh = 0, U = 0, nruns = 0;
    long long ncells = 0;
    const double* u = nullptr;          // [48] Gauss-Hermite nodes
    const double* w = nullptr;          // [48] stationary weights
    const double* K = nullptr;          // [(nsh - 1) * 48 * 48] transition matrices K[s][i][j]
    const double* ku = nullptr;         // [U] unique cell kappa
    const double* gu = nullptr;         // [U] unique cell gamma
    const int* cu = nullptr;            // [ncells] unique-cell index, run-sorted
    const double2* wab = nullptr;       // [ncells] (w a, w b)
    const float2* wabf = nullptr;       // [ncells] the same, rounded to FP32
    const long long* run_cell = nullptr;   // [nruns + 1] cell offsets
    const int* run_kind = nullptr;      // [nruns] 0 linear, 1 left (states lo..47), 2 right (states 0..hi)
    const int* run_bound = nullptr;     // [nruns] lo (left) or hi (right)
    const int* sh_run = nullptr;        // [nsh + 1] run offsets
};
size_t vp_table_bytes(int precision, int U, int nk, int nq);
int vp_rows_per_pass(int nsh, int nk, int nq, size_t z_cap_bytes);
void launch_vp_lnR(int precision, const VpDevice& d, const double* kv, int nk, const double* qv, int nq, void* tables,
                   double2* zbuf, int rows_per_pass, double* out_re, double* out_im, cudaStream_t st, int npieces = 1);
// pieces per shell for the phase-1 kernel so that a small point grid still fills the GPU
int vp_pieces(int nsh, int rows, int nq);

// ---- 1-D CF sweep and FMA probes
int sweep1d_chunks(int nk, long long nc);
void launch_sweep1d(int precision, const double* kk, int nk, const double* kap, const double* w, const float* kh,
                    const float* kl, const float* wf, long long nc, int nchunks, double2* part, double* re,
                    double* im, cudaStream_t st);
void launch_fma_probe(int fp64, void* out, int blocks, int iters, cudaStream_t st);

// ---- binned-cell deposit of the population build (cells.cu)
struct CellsGeom {                        // the lattices: edge counts and the parameters of the log bin guess
    int nekf, negf, nekc, negc;           // edges, stored [ekf | egf | ekc | egc]
    double kf_lo, kf_dl, gf_lo, gf_dl, kc_lo, kc_dl, gc_lo, gc_dl;
    double g_clip, k_max_fine;            // gamma clipped below at g_clip; |kappa| < k_max_fine enters lin
    int nord;
};
int cells_edge_smem_bytes(const CellsGeom& g);
void launch_cells_hist(const CellsGeom& g, const double* edges, long long n, const double* K, const double* Gm,
                       const double* W, const long long* off, int n_obj, const int* shell, const double* betas,
                       double* H0, double* H0k, double* H0g, double* Hc, double* sums, int n_sm, cudaStream_t st);
constexpr int kXiChunk = 1024;            // points of one object per xi work item
constexpr int kCellsXiMaxEdges = 1024;    // coarse kappa + gamma edges the xi kernel holds in shared memory
struct CellsXiItem { long long first; int count, obj; };
void launch_cells_xi(const CellsGeom& g, const double* edges, const CellsXiItem* items, int n_items,
                     const double* K, const double* Gm, const double* W, const double* R, const double* beta,
                     const unsigned char* tang, const double* kp, int nkp, int mm, double* Hx, double* lx, double* Wb,
                     cudaStream_t st);
void launch_cells_xi_tail(const double* kp, int nkp, double coef, double Rm, double* lx, cudaStream_t st);
void launch_cells_xi_flags(const double* Hx, int nbins, int mm, int nkp, unsigned char* flags, cudaStream_t st);
void launch_cells_xi_rows(const double* Hx, int mm, int nkp, int m, const int* idx, int nidx, const double* cen,
                          int ngc, int cen_axis, const double* lxm, const double* sw, double* A, cudaStream_t st);
int cells_gram_parts(long long nrows, int chunk);
void launch_cells_gram(const double* A, long long nrows, int nkp, int chunk, double* part, double* Gram, cudaStream_t st);
void launch_cells_project(const double* A, long long nrows, int nkp, const double* V, int nkeep, double* rows,
                          cudaStream_t st);

}  // namespace sgl
