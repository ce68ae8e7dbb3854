// Per-cosmology tables (sgl_cosmo_tables): validation of the reference's cosmology domain
// (pipeline.py:39-79, sgl.py:68-160) and the launch of cosmo.cu's one-CTA-per-cosmology kernel.
#include <algorithm>
#include <numeric>

#include "host.cuh"

extern "C" {

sgl_status sgl_cosmo_tables(sgl_ctx* ctx, int n, const double* params, int nz, const double* z, int nm, const double* M,
                            int nzm, const double* zm, double* E, double* chi, double* DM, double* D, double* sigmaM,
                            double* dlnsig, double* dndlnM, double* conc) {
    if (!ctx) return SGL_ERR_VALUE;
    if (n < 1 || !params || nz < 1 || !z || nm < 1 || !M || nzm < 0 || (nzm > 0 && !zm) || !E || !chi || !DM || !D ||
        !sigmaM || !dlnsig || (nzm > 0 && (!dndlnM || !conc)))
        return fail(ctx, SGL_ERR_VALUE, "sgl_cosmo_tables: invalid sizes or NULL arrays");
    for (int j = 0; j < nz; ++j)
        if (!(z[j] >= 0) || z[j] > 1e6 || (j > 0 && !(z[j] > z[j - 1])))
            return fail(ctx, SGL_ERR_VALUE, "sgl_cosmo_tables: z must be ascending in [0, 1e6]");
    for (int j = 0; j < nzm; ++j)
        if (!(zm[j] >= 0) || zm[j] > 1e6) return fail(ctx, SGL_ERR_VALUE, "sgl_cosmo_tables: mass-function z outside [0, 1e6]");
    for (int j = 0; j < nm; ++j)
        if (!(M[j] > 0) || !std::isfinite(M[j])) return fail(ctx, SGL_ERR_VALUE, "sgl_cosmo_tables: masses must be positive");
    for (int i = 0; i < n; ++i) {
        const double* p = params + 9LL * i;
        const double h = p[0], Om = p[1], Ob = p[2], s8 = p[3], ns = p[4], zeq = p[5], Ok = p[6], w0 = p[7], wa = p[8];
        const std::string who = "cosmology " + std::to_string(i) + ": ";
        for (int q = 0; q < 6; ++q)
            if (!std::isfinite(p[q]) || !(p[q] > 0)) return fail(ctx, SGL_ERR_VALUE, who + "h, Om, Ob, s8, ns, zeq must be finite positive numbers");
        if (!std::isfinite(Ok) || !std::isfinite(w0) || !std::isfinite(wa)) return fail(ctx, SGL_ERR_VALUE, who + "Ok, w0, wa must be finite");
        if (!(Ob < Om && Om <= 1)) return fail(ctx, SGL_ERR_VALUE, who + "require 0 < Ob < Om <= 1");
        if (!(w0 >= -2.0 && w0 <= 1.0)) return fail(ctx, SGL_ERR_VALUE, who + "dark energy requires -2 <= w0 <= 1");
        if (!(w0 + wa < 0.0)) return fail(ctx, SGL_ERR_VALUE, who + "dark energy requires w0 + wa < 0");
        const double Or = Om / (1.0 + zeq), OL = 1.0 - Om - Ok - Or;
        const double de_m = OL / Om * std::pow(1101.0, 3 * (w0 + wa)) * std::exp(-3 * wa * 1100.0 / 1101.0);
        if (de_m > 1e-2) return fail(ctx, SGL_ERR_VALUE, who + "dark energy exceeds 1e-2 of the matter density at z = 1100");
        for (int q = 0; q < 4096; ++q) {
            const double a = std::pow(10.0, -6.0 + 6.0 * q / 4095.0), zp1 = 1.0 / a;
            const double de = OL * std::pow(zp1, 3 * (1 + w0 + wa)) * std::exp(-3 * wa * (1 - a));
            if (!(Om * zp1 * zp1 * zp1 + Or * zp1 * zp1 * zp1 * zp1 + Ok * zp1 * zp1 + de > 0))
                return fail(ctx, SGL_ERR_VALUE, who + "E(z)^2 <= 0 somewhere in 0 <= z <= 1e6");
        }
        (void)s8; (void)ns; (void)h;
    }
    CK(cudaSetDevice(ctx->device));
    // growth outputs: every z and every mass-function z, ascending in ln a
    const int nx = nz + nzm;
    std::vector<double> xs((size_t)nx);
    for (int j = 0; j < nz; ++j) xs[(size_t)j] = -std::log1p(z[j]);
    for (int j = 0; j < nzm; ++j) xs[(size_t)nz + j] = -std::log1p(zm[j]);
    std::vector<int> order((size_t)nx);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return xs[(size_t)a] < xs[(size_t)b]; });
    std::vector<double> x_out((size_t)nx);
    for (int j = 0; j < nx; ++j) x_out[(size_t)j] = xs[(size_t)order[(size_t)j]];
    const double A_st = 1.0 / (1.0 + std::pow(2.0, -0.3) * std::tgamma(0.5 - 0.3) / std::sqrt(M_PI));
    const long long nzmm = std::max(1, nzm);
    DBUF(d_p, double, "cos_params", 9LL * n);
    DBUF(d_z, double, "cos_z", nz);
    DBUF(d_x, double, "cos_x", nx);
    DBUF(d_slot, int, "cos_slot", nx);
    DBUF(d_M, double, "cos_M", nm);
    DBUF(d_zm, double, "cos_zm", nzmm);
    DBUF(d_E, double, "cos_E", (long long)n * nz);
    DBUF(d_chi, double, "cos_chi", (long long)n * nz);
    DBUF(d_DM, double, "cos_DM", (long long)n * nz);
    DBUF(d_D, double, "cos_D", (long long)n * nz);
    DBUF(d_Dm, double, "cos_Dm", (long long)n * nzmm);
    DBUF(d_sig, double, "cos_sig", (long long)n * nm);
    DBUF(d_dls, double, "cos_dls", (long long)n * nm);
    DBUF(d_dn, double, "cos_dn", (long long)n * nzmm * nm);
    DBUF(d_cc, double, "cos_conc", (long long)n * nzmm * nm);
    DBUF(d_work, double, "cos_work", (long long)n * cosmo_work_doubles(nx));
    CKS(upload(ctx, d_p, params, 9 * (size_t)n));
    CKS(upload(ctx, d_z, z, (size_t)nz));
    CKS(upload(ctx, d_x, x_out.data(), x_out.size()));
    CKS(upload(ctx, d_slot, order.data(), order.size()));
    CKS(upload(ctx, d_M, M, (size_t)nm));
    if (nzm > 0) CKS(upload(ctx, d_zm, zm, (size_t)nzm));
    launch_cosmo_tables(n, d_p, nz, d_z, d_x, d_slot, nx, nm, d_M, nzm, d_zm, A_st, d_E, d_chi, d_DM, d_D, d_Dm, d_sig,
                        d_dls, d_dn, d_cc, d_work, ctx->stream);
    CKLAUNCH();
    const cudaStream_t st = ctx->stream;
    CK(cudaMemcpyAsync(E, d_E, sizeof(double) * n * nz, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(chi, d_chi, sizeof(double) * n * nz, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(DM, d_DM, sizeof(double) * n * nz, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(D, d_D, sizeof(double) * n * nz, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(sigmaM, d_sig, sizeof(double) * n * nm, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(dlnsig, d_dls, sizeof(double) * n * nm, cudaMemcpyDeviceToHost, st));
    if (nzm > 0) {
        CK(cudaMemcpyAsync(dndlnM, d_dn, sizeof(double) * n * nzm * nm, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(conc, d_cc, sizeof(double) * n * nzm * nm, cudaMemcpyDeviceToHost, st));
    }
    CKS(sync_stream(ctx));
    for (long long e = 0; e < (long long)n * nz; ++e)
        if (!std::isfinite(chi[e]) || !std::isfinite(D[e])) return fail(ctx, SGL_ERR_NONFINITE, "cosmology tables are not finite");
    return SGL_OK;
}

}  // extern "C"
