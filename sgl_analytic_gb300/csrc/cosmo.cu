// Per-cosmology background and linear-theory tables on the GPU: the default chain's Cosmology of the
// reference (sgl.py:65-640 as pipeline.make_cosmology builds it, pipeline.py:39-79): CPL dark energy
// with curvature and radiation Omega_r = Om / (1 + z_eq); E(z); the radial comoving distance chi(z) and
// the transverse D_M(z); the linear growth D(z) from the growth ODE (sgl.py:310-347); the EH98 transfer
// function with baryons (sgl.py:391-445); sigma(M) through the smooth-k filter with the top-hat sigma_8
// anchor (sgl.py:452-553) on the reference's k and M grids with its not-a-knot spline in ln M; the
// Sheth-Tormen dn/dln M (sgl.py:556-568) and the Ludlow+16 concentration (sgl.py:570-606).
//
// One CTA per cosmology.  The arithmetic is the reference's (FP64); where it calls an adaptive
// integrator this file uses fixed high-order rules instead: composite 8-point Gauss-Legendre panels
// of width <= 0.02 for chi (the reference: quad), classical RK4 with 2^15 steps in ln a for the growth
// ODE (the reference: DOP853 at rtol 2e-10), and the not-a-knot cubic spline through its tridiagonal
// system solved by elimination (the reference: scipy's CubicSpline / solve_banded).
#include "common.cuh"
#include "kernels.cuh"

namespace sgl {
namespace {

constexpr double kCkms = 299792.458;          // km/s
constexpr double kRhoc0Unit = 2.77536627e11;  // Msun / Mpc^3 / h^2
constexpr double kTcmb = 2.7255;
constexpr double kDc = 1.686;
constexpr int kNk = 4000;                      // sigma(R) k grid: logspace(-5, 3, 4000)
constexpr int kNm = 500;                       // sigma(M) spline nodes: logspace(4, 17, 500)
constexpr int kOdeSteps = 1 << 15;
constexpr int kThreads = 256;

struct Cos {
    double h, Om, Ob, s8, ns, zeq, Ok, w0, wa;
    double Or, OL, H0, rhom;
};

__device__ __forceinline__ Cos make_cos(const double* p) {
    Cos c;
    c.h = p[0]; c.Om = p[1]; c.Ob = p[2]; c.s8 = p[3]; c.ns = p[4]; c.zeq = p[5]; c.Ok = p[6]; c.w0 = p[7]; c.wa = p[8];
    c.Or = c.Om / (1.0 + c.zeq);
    c.OL = 1.0 - c.Om - c.Ok - c.Or;
    c.H0 = 100.0 * c.h;
    c.rhom = c.Om * kRhoc0Unit * c.h * c.h;
    return c;
}

// E(z), the reference's branches (sgl.py:183-195)
__device__ double cos_E(const Cos& c, double z) {
    if (c.w0 == -1.0 && c.wa == 0.0 && c.Ok == 0.0)
        return sqrt(c.Om * (1 + z) * (1 + z) * (1 + z) + c.Or * (1 + z) * (1 + z) * (1 + z) * (1 + z) + c.OL);
    const double zp1 = 1.0 + z;
    double de;
    if (c.wa == 0.0) de = c.w0 == -1.0 ? c.OL : c.OL * pow(zp1, 3 * (1 + c.w0));
    else de = c.OL * pow(zp1, 3 * (1 + c.w0 + c.wa)) * exp(-3 * c.wa * (1 - 1 / zp1));
    return sqrt(c.Om * zp1 * zp1 * zp1 + c.Or * zp1 * zp1 * zp1 * zp1 + c.Ok * zp1 * zp1 + de);
}

// transverse comoving distance of a radial interval (sgl.py:219-238)
__device__ double cos_fK(const Cos& c, double chi) {
    if (c.Ok == 0.0) return chi;
    const double u = chi * c.H0 / kCkms;
    const double t = c.Ok * u * u;
    if (fabs(t) < 1e-5) return chi * (1 + t / 6 + t * t / 120 + t * t * t / 5040);
    const double x = sqrt(fabs(c.Ok)) * u;
    return chi * (c.Ok > 0 ? sinh(x) / x : sin(x) / x);
}

// the growth ODE's right-hand side in x = ln a (sgl.py:320-336)
__device__ __forceinline__ void growth_rhs(const Cos& c, double x, double y0, double y1, double& d0, double& d1) {
    const double matter = c.Om * exp(-3 * x);
    const double a = exp(x);
    const double de = c.OL * exp(-3 * (1 + c.w0 + c.wa) * x + 3 * c.wa * (a - 1));
    const double wz = c.w0 + c.wa * (1 - a);
    const double curvature = c.Ok * exp(-2 * x);
    double total, dh;
    if (c.Or != 0.0) {
        const double rad = c.Or * exp(-4 * x);
        total = matter + rad + curvature + de;
        dh = -0.5 * (3 * matter + 4 * rad + 2 * curvature + 3 * (1 + wz) * de) / total;
    } else {
        total = matter + curvature + de;
        dh = -0.5 * (3 * matter + 2 * curvature + 3 * (1 + wz) * de) / total;
    }
    d0 = y1;
    d1 = -(2 + dh) * y1 + 1.5 * (matter / total) * y0;
}

__device__ __forceinline__ void rk4(const Cos& c, double x, double hs, double& y0, double& y1) {
    double a0, a1, b0, b1, c0, c1, e0, e1;
    growth_rhs(c, x, y0, y1, a0, a1);
    growth_rhs(c, x + 0.5 * hs, y0 + 0.5 * hs * a0, y1 + 0.5 * hs * a1, b0, b1);
    growth_rhs(c, x + 0.5 * hs, y0 + 0.5 * hs * b0, y1 + 0.5 * hs * b1, c0, c1);
    growth_rhs(c, x + hs, y0 + hs * c0, y1 + hs * c1, e0, e1);
    y0 += hs / 6 * (a0 + 2 * b0 + 2 * c0 + e0);
    y1 += hs / 6 * (a1 + 2 * b1 + 2 * c1 + e1);
}

// EH98 CDM + baryon transfer function (sgl.py:391-445; Eisenstein & Hu 1998, ApJ 496, 605)
struct Eh98 {
    double Om, Ob, Oc, keq, ksilk, ac, bc, s, ab, bb, bnode;
};

__device__ Eh98 make_eh98(const Cos& c) {
    Eh98 e;
    const double h = c.h, Om = c.Om, Ob = c.Ob, Oc = Om - Ob;
    const double wm = Om * h * h, wb = Ob * h * h;
    e.Om = Om; e.Ob = Ob; e.Oc = Oc;
    e.keq = (c.H0 / kCkms) * sqrt(2.0 * Om) * sqrt(1.0 + c.zeq);
    e.ksilk = 0.0016 * pow(wb, 0.52) * pow(wm, 0.73) * (1 + pow(10.4 * wm, -0.95));
    const double a1 = pow(46.9 * wm, 0.67) * (1 + pow(32.1 * wm, -0.532));
    const double a2 = pow(12.0 * wm, 0.424) * (1 + pow(45.0 * wm, -0.582));
    const double b1 = 0.944 / (1 + pow(458 * wm, -0.708));
    const double b2 = pow(0.395 * wm, -0.026);
    e.ac = pow(a1, -Ob / Om) * pow(a2, -pow(Ob / Om, 3));
    e.bc = 1.0 / (1 + b1 * (pow(Oc / Om, b2) - 1));
    e.s = 44.5 * log(9.83 / wm) / sqrt(1 + 10 * pow(wb, 0.75));
    const double b3 = 0.313 * pow(wm, -0.419) * (1 + 0.607 * pow(wm, 0.674));
    const double b4 = 0.238 * pow(wm, 0.223);
    const double zd = 1291 * pow(wm, 0.251) / (1 + 0.659 * pow(wm, 0.828)) * (1 + b3 * pow(wb, b4));
    const double Rd = 31.5 * wb * pow(kTcmb / 2.7, -4) / (zd / 1000.0);
    const double y = (1 + c.zeq) / (1 + zd);
    const double g2 = y * (-6 * sqrt(1 + y) + (2.0 + 3.0 * y) * log((sqrt(1 + y) + 1) / (sqrt(1 + y) - 1)));
    e.ab = 2.07 * e.keq * e.s * pow(1 + Rd, -0.75) * g2;
    e.bb = 0.5 + Ob / Om + (3.0 - 2.0 * Ob / Om) * sqrt(1 + (17.2 * wm) * (17.2 * wm));
    e.bnode = 8.41 * pow(wm, 0.435);
    return e;
}

__device__ __forceinline__ double eh_To1(const Eh98& e, double k, double a_c, double b_c) {
    const double qq = k / (13.41 * e.keq);
    const double C1 = 14.2 / a_c + 386.0 / (1 + 69.9 * pow(qq, 1.08));
    const double num = log(M_E + 1.8 * b_c * qq);
    return num / (num + C1 * qq * qq);
}

__device__ double eh_T(const Eh98& e, double k) {
    const double ks = k * e.s;
    const double fk = 1.0 / (1 + pow(ks / 5.4, 4));
    const double TC = fk * eh_To1(e, k, 1.0, e.bc) + (1 - fk) * eh_To1(e, k, e.ac, e.bc);
    const double s3 = e.s / cbrt(1 + pow(e.bnode / ks, 3));
    const double x = k * s3;
    const double jo = x < 1e-8 ? 1.0 - x * x / 6.0 : sin(x) / x;
    const double TB = (eh_To1(e, k, 1.0, 1.0) / (1 + (ks / 5.2) * (ks / 5.2)) +
                       e.ab / (1 + pow(e.bb / ks, 3)) * exp(-pow(k / e.ksilk, 1.4))) * jo;
    return e.Ob / e.Om * TB + e.Oc / e.Om * TC;
}

// block-wide sum of one value per thread
__device__ double block_sum(double v, double* red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0) {
        for (int w = 0; w < kThreads / 32; ++w) t += red[w];
        red[kThreads / 32] = t;
    }
    __syncthreads();
    return red[kThreads / 32];
}

struct CosArgs {
    const double* params;                 // [cosmology][9]
    int nz; const double* z;              // distance / growth redshifts (ascending)
    const double* x_out;                  // growth output points ln a, ascending, with their slots
    const int* x_slot; int nx;
    int nm; const double* M;              // output masses
    int nzm; const double* zm;            // mass-function redshifts
    double A_st;                          // Sheth-Tormen normalisation
    double* E; double* chi; double* DM; double* D;       // [cosmology][nz]
    double* Dm;                           // [cosmology][nzm] growth at the mass-function redshifts
    double* sigM; double* dlnsig;         // [cosmology][nm] sigma(M, 0), d ln sigma / d ln M
    double* dndlnM; double* conc;         // [cosmology][nzm][nm]
    double* work;                         // [cosmology][work_stride] scratch
    long long work_stride;                // 2 kNk + 3 kNm + nx
};

__global__ void __launch_bounds__(kThreads) k_cosmo_tables(CosArgs a) {
    __shared__ double red[kThreads / 32 + 1];
    __shared__ double s_anorm, s_D0;
    const int ci = blockIdx.x;
    const Cos c = make_cos(a.params + 9LL * ci);
    double* kP = a.work + (long long)ci * a.work_stride;          // k^2 P_shape at the k grid
    double* kg = kP + kNk;                                        // the k grid
    double* lnM = kg + kNk;                                       // spline nodes, values, slopes
    double* lns = lnM + kNm;
    double* sl = lns + kNm;
    double* sc = sl + kNm;                                        // growth ODE at the output points
    const int t = threadIdx.x;
    // ---- growth ODE (one thread; the others proceed with sigma(M) meanwhile)
    if (t == 0) {
        const double x0 = log(1e-6);
        double y0 = exp(x0) + (c.Or != 0.0 ? (2.0 / 3.0) * c.Or / c.Om : 0.0), y1 = exp(x0);
        const double hs = -x0 / kOdeSteps;
        double x = x0;
        int j = 0;
        for (int s = 0; s < kOdeSteps; ++s) {
            const double xn = s == kOdeSteps - 1 ? 0.0 : x0 + (s + 1) * hs;
            while (j < a.nx && a.x_out[j] <= xn) {       // an output inside this step: a partial step to it
                double u0 = y0, u1 = y1;
                if (a.x_out[j] > x) rk4(c, x, a.x_out[j] - x, u0, u1);
                sc[j] = u0;
                ++j;
            }
            rk4(c, x, xn - x, y0, y1);
            x = xn;
        }
        for (; j < a.nx; ++j) sc[j] = y0;
        s_D0 = y0;
    }
    // ---- k grid, transfer function, sigma_8 anchor through the real-space top hat
    const Eh98 e = make_eh98(c);
    for (int i = t; i < kNk; i += kThreads) {
        const double k = pow(10.0, -5.0 + i * (8.0 / (kNk - 1)));
        kg[i] = i == kNk - 1 ? 1000.0 : k;
        const double T = eh_T(e, kg[i]);
        kP[i] = kg[i] * kg[i] * pow(kg[i], c.ns) * T * T;
    }
    __syncthreads();
    {
        const double R = 8.0 / c.h;
        double acc = 0.0;
        for (int i = t; i < kNk - 1; i += kThreads) {
            double W[2];
            for (int q = 0; q < 2; ++q) {
                const double x = kg[i + q] * R;
                W[q] = 3 * (sin(x) - x * cos(x)) / (x * x * x);
            }
            acc += 0.5 * (kP[i] * W[0] * W[0] + kP[i + 1] * W[1] * W[1]) * (kg[i + 1] - kg[i]);
        }
        const double s2 = block_sum(acc, red);
        if (t == 0) s_anorm = c.s8 / sqrt(s2 / (2 * M_PI * M_PI));
    }
    __syncthreads();
    // ---- ln sigma(M) on the spline nodes (smooth-k filter), one warp per node
    const int warp = t >> 5, lane = t & 31;
    for (int m = warp; m < kNm; m += kThreads / 32) {
        const double Mn = pow(10.0, 4.0 + m * (13.0 / (kNm - 1)));
        const double R = cbrt(3 * Mn / (4 * M_PI * c.rhom));
        double acc = 0.0;
        for (int i = lane; i < kNk - 1; i += 32) {
            const double x0 = 0.43 * kg[i] * R, x1 = 0.43 * kg[i + 1] * R;
            const double W0 = 1.0 / (1.0 + pow(x0, 6)), W1 = 1.0 / (1.0 + pow(x1, 6));
            acc += 0.5 * (kP[i] * W0 * W0 + kP[i + 1] * W1 * W1) * (kg[i + 1] - kg[i]);
        }
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) {
            lnM[m] = log(m == kNm - 1 ? 1e17 : Mn);
            lns[m] = log(s_anorm * sqrt(acc / (2 * M_PI * M_PI)));
        }
    }
    __syncthreads();
    // ---- the not-a-knot spline's slopes: tridiagonal system, forward elimination and back substitution
    if (t == 0) {
        const int n = kNm;
        double* dg = kP;                       // the k-grid scratch is free now: diagonal, upper, rhs
        double* up = kP + n;
        double* rhs = kP + 2 * n;
        double* lo = kP + 3 * n;
        for (int i = 1; i < n - 1; ++i) {
            const double dx0 = lnM[i] - lnM[i - 1], dx1 = lnM[i + 1] - lnM[i];
            const double m0 = (lns[i] - lns[i - 1]) / dx0, m1 = (lns[i + 1] - lns[i]) / dx1;
            lo[i] = dx1;
            dg[i] = 2 * (dx0 + dx1);
            up[i] = dx0;
            rhs[i] = 3 * (dx1 * m0 + dx0 * m1);
        }
        {
            const double dx0 = lnM[1] - lnM[0], dx1 = lnM[2] - lnM[1], d = lnM[2] - lnM[0];
            const double m0 = (lns[1] - lns[0]) / dx0, m1 = (lns[2] - lns[1]) / dx1;
            dg[0] = dx1;
            up[0] = d;
            rhs[0] = ((dx0 + 2 * d) * dx1 * m0 + dx0 * dx0 * m1) / d;
        }
        {
            const double dx0 = lnM[n - 2] - lnM[n - 3], dx1 = lnM[n - 1] - lnM[n - 2], d = lnM[n - 1] - lnM[n - 3];
            const double m0 = (lns[n - 2] - lns[n - 3]) / dx0, m1 = (lns[n - 1] - lns[n - 2]) / dx1;
            dg[n - 1] = dx0;
            lo[n - 1] = d;
            rhs[n - 1] = (dx1 * dx1 * m0 + (2 * d + dx1) * dx0 * m1) / d;
        }
        for (int i = 1; i < n; ++i) {
            const double f = lo[i] / dg[i - 1];
            dg[i] -= f * up[i - 1];
            rhs[i] -= f * rhs[i - 1];
        }
        sl[n - 1] = rhs[n - 1] / dg[n - 1];
        for (int i = n - 2; i >= 0; --i) sl[i] = (rhs[i] - up[i] * sl[i + 1]) / dg[i];
    }
    // ---- distances: 8-point Gauss-Legendre panels of width <= 0.02 between consecutive redshifts
    for (int j = t; j < a.nz; j += kThreads) {
        const double za = j == 0 ? 0.0 : a.z[j - 1], zb = a.z[j];
        const int np = max(1, (int)ceil((zb - za) / 0.02));
        const double xg[4] = {0.1834346424956498, 0.5255324099163290, 0.7966664774136267, 0.9602898564975363};
        const double wg[4] = {0.3626837833783620, 0.3137066458778873, 0.2223810344533745, 0.1012285362903763};
        const double hw = 0.5 * (zb - za) / np;
        double acc = 0.0;
        for (int q = 0; q < np; ++q) {
            const double mid = za + (2 * q + 1) * hw;
            for (int g = 0; g < 4; ++g)
                acc += wg[g] * (1.0 / cos_E(c, mid - hw * xg[g]) + 1.0 / cos_E(c, mid + hw * xg[g]));
        }
        a.chi[(long long)ci * a.nz + j] = acc * hw * kCkms / c.H0;          // this interval; summed below
        a.E[(long long)ci * a.nz + j] = cos_E(c, zb);
    }
    __syncthreads();
    if (t == 0) {
        double run = 0.0;
        for (int j = 0; j < a.nz; ++j) {
            run += a.chi[(long long)ci * a.nz + j];
            a.chi[(long long)ci * a.nz + j] = run;
            a.DM[(long long)ci * a.nz + j] = cos_fK(c, run);
        }
        for (int j = 0; j < a.nx; ++j) {
            const int slot = a.x_slot[j];
            const double Dv = sc[j] / s_D0;
            if (slot < a.nz) a.D[(long long)ci * a.nz + slot] = Dv;
            else a.Dm[(long long)ci * a.nzm + (slot - a.nz)] = Dv;
        }
    }
    __syncthreads();
    // ---- sigma(M), the mass function and the concentration at the output masses
    for (int e2 = t; e2 < a.nm; e2 += kThreads) {
        const double x = log(a.M[e2]);
        int lo = 0, hi = kNm - 2;                       // the spline interval holding x (clamped)
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (lnM[mid] <= x) lo = mid; else hi = mid - 1;
        }
        const double dx = lnM[lo + 1] - lnM[lo];
        const double slope = (lns[lo + 1] - lns[lo]) / dx;
        const double tt = (sl[lo] + sl[lo + 1] - 2 * slope) / dx;
        const double c0 = tt / dx, c1 = (slope - sl[lo]) / dx - tt, c2 = sl[lo], c3 = lns[lo];
        const double u = x - lnM[lo];
        const double lnsig = ((c0 * u + c1) * u + c2) * u + c3;
        const double dls = (3 * c0 * u + 2 * c1) * u + c2;
        const double sig0 = exp(lnsig);
        a.sigM[(long long)ci * a.nm + e2] = sig0;
        a.dlnsig[(long long)ci * a.nm + e2] = dls;
        for (int q = 0; q < a.nzm; ++q) {
            const double zq = a.zm[q];
            const double sig = sig0 * a.Dm[(long long)ci * a.nzm + q];
            const double nu = (kDc / sig) * (kDc / sig);
            const double qn = 0.8 * nu;
            const double mult = a.A_st * (1 + pow(qn, -0.3)) * sqrt(qn / (2 * M_PI)) * exp(-qn / 2);
            a.dndlnM[((long long)ci * a.nzm + q) * a.nm + e2] = (c.rhom / a.M[e2]) * mult * (-2 * dls);
            const double zc = zq > 7.0 ? 7.0 : zq;
            const double ap = 1.0 + zc;
            const double poly = 4.135 - 0.564 * ap - 0.210 * ap * ap + 0.0557 * ap * ap * ap - 0.00348 * ap * ap * ap * ap;
            const double qc = kDc / (sig0 * poly);
            const double cc0 = 3.395 * pow(ap, -0.215), beta = 0.307 * pow(ap, 0.540);
            const double g1 = 0.628 * pow(ap, -0.047), g2 = 0.317 * pow(ap, -0.893);
            a.conc[((long long)ci * a.nzm + q) * a.nm + e2] = cc0 * pow(qc, -g1) * pow(1.0 + pow(qc, 1.0 / beta), -beta * (g2 - g1));
        }
    }
}

}  // namespace

long long cosmo_work_doubles(int nx) { return 2LL * kNk + 3LL * kNm + nx; }

void launch_cosmo_tables(int n, const double* params, int nz, const double* z, const double* x_out, const int* x_slot,
                         int nx, int nm, const double* M, int nzm, const double* zm, double A_st, double* E,
                         double* chi, double* DM, double* D, double* Dm, double* sigM, double* dlnsig,
                         double* dndlnM, double* conc, double* work, cudaStream_t st) {
    CosArgs a{params, nz, z, x_out, x_slot, nx, nm, M, nzm, zm, A_st, E, chi, DM, D, Dm, sigM, dlnsig, dndlnM, conc,
              work, cosmo_work_doubles(nx)};
    k_cosmo_tables<<<n, kThreads, 0, st>>>(a);
    SGL_COUNT(1);
}

}  // namespace sgl
