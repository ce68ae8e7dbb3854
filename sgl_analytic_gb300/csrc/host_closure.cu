// Set-up of the positive (vp) Cox closure from its per-shell population: the latent chain, the
// per-group rates calibrated to the population's kappa clustering variance, the unique cells and
// the rate intervals, then the same installation as sgl_vp_set.
//
// Restates, in this order (reference sgl_analytic v0.2.0):
//   Closure.__init__            pos_closure.py:453-491  (states, transitions, groups, unique cells)
//   Closure.variance/calibrate  pos_closure.py:561-591  (chain variance, Brent root in ln eta)
//   transition                  pos_closure.py:251-267  (stationary-balanced Gaussian-copula kernel)
//   vp_rates / group_rates      pos_closure.py:273-318
//   chain_variance              pos_closure.py:352-369
//   Closure._blocked_setup      pos_closure.py:493-514  (cells by group, group offsets per shell)
//   FusedVP / rate_intervals    pos_closure_fused.py:18-48, 58-67
// and numpy.polynomial.hermite_e.hermegauss for the 48 latent states.  The per-shell population
// itself (pos_closure.population, pos_closure.py:388-450: the cells of each shell with their
// loadings phi, the line-of-sight correlations rho between shells, f_var and the kappa / gamma
// variance targets) is this entry point's input.
#include <cmath>
#include <limits>
#include <numeric>

#include "host.cuh"

namespace sglh {
namespace {

// ---- Gauss-Hermite (probabilists') rule on n states --------------------------------------
// the degree-n normalised Hermite_e polynomial at x by its three-term recurrence (the form numpy
// uses for the Gauss points: no overflow at high degree)
double normed_hermite_e(double x, int n) {
    const double c00 = 1.0 / std::sqrt(std::sqrt(2.0 * M_PI));
    if (n == 0) return c00;
    double c0 = 0.0, c1 = c00, nd = (double)n;
    for (int i = 0; i < n - 1; ++i) {
        const double tmp = c0;
        c0 = -c1 * std::sqrt((nd - 1.0) / nd);
        c1 = tmp + c1 * x * std::sqrt(1.0 / nd);
        nd = nd - 1.0;
    }
    return c0 + c1 * x;
}

// nodes: eigenvalues of the symmetric Jacobi matrix (zero diagonal, off-diagonal sqrt(k)) by
// bisection on Sturm counts, then one Newton step; weights 1 / He~_{n-1}(x)^2 (scaled), both
// symmetrised; weights normalised to sum 1 (the closure's stationary distribution)
void hermegauss(int n, std::vector<double>& x, std::vector<double>& w) {
    x.assign((size_t)n, 0.0);
    w.assign((size_t)n, 0.0);
    const double R = 2.0 * std::sqrt((double)n) + 1.0;
    auto count_below = [&](double lam) {              // eigenvalues < lam
        int cnt = 0;
        double q = -lam;
        if (q < 0) ++cnt;
        for (int i = 1; i < n; ++i) {
            const double qq = q == 0.0 ? 1e-300 : q;
            q = -lam - (double)i / qq;                 // off-diagonal sqrt(i) squared
            if (q < 0) ++cnt;
        }
        return cnt;
    };
    for (int k = 0; k < n; ++k) {
        double lo = -R, hi = R;
        for (int it = 0; it < 200 && hi - lo > 0; ++it) {
            const double mid = 0.5 * (lo + hi);
            if (mid <= lo || mid >= hi) break;
            if (count_below(mid) > k) hi = mid; else lo = mid;
        }
        x[(size_t)k] = 0.5 * (lo + hi);
    }
    for (int k = 0; k < n; ++k) {
        const double dy = normed_hermite_e(x[(size_t)k], n);
        const double df = normed_hermite_e(x[(size_t)k], n - 1) * std::sqrt((double)n);
        x[(size_t)k] -= dy / df;
    }
    std::vector<double> fm((size_t)n);
    double fmax = 0.0;
    for (int k = 0; k < n; ++k) { fm[(size_t)k] = normed_hermite_e(x[(size_t)k], n - 1); fmax = std::max(fmax, std::fabs(fm[(size_t)k])); }
    for (int k = 0; k < n; ++k) { const double f = fm[(size_t)k] / fmax; w[(size_t)k] = 1.0 / (f * f); }
    std::vector<double> ws(w), xs(x);
    for (int k = 0; k < n; ++k) {
        w[(size_t)k] = (ws[(size_t)k] + ws[(size_t)(n - 1 - k)]) / 2.0;
        x[(size_t)k] = (xs[(size_t)k] - xs[(size_t)(n - 1 - k)]) / 2.0;
    }
    double s = 0.0;
    for (double v : w) s += v;
    const double sc = std::sqrt(2.0 * M_PI) / s;
    for (double& v : w) v *= sc;
    s = 0.0;
    for (double v : w) s += v;
    for (double& v : w) v /= s;
}

// ---- transition kernel between consecutive shells ------------------------------------------
// J_ij = w_i w_j exp((2 rho x y - rho^2 (x^2 + y^2)) / (2 (1 - rho^2))), balanced symmetrically
// (v <- v sqrt(w / (v J v))) until w is stationary to 3e-14; K = v_i J_ij v_j / w_i
bool transition(const std::vector<double>& u, const std::vector<double>& w, double rho, double* K) {
    const int n = (int)u.size();
    std::vector<double> J((size_t)n * n), v((size_t)n, 1.0), Jv((size_t)n), marg((size_t)n);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            const double x = u[(size_t)i], y = u[(size_t)j];
            const double lr = (2 * rho * x * y - rho * rho * (x * x + y * y)) / (2 * (1 - rho * rho));
            J[(size_t)i * n + j] = w[(size_t)i] * w[(size_t)j] * std::exp(lr);
        }
    bool conv = false;
    for (int it = 0; it < 10000; ++it) {
        double err = 0.0;
        for (int i = 0; i < n; ++i) {
            double s = 0.0;
            for (int j = 0; j < n; ++j) s += J[(size_t)i * n + j] * v[(size_t)j];
            marg[(size_t)i] = v[(size_t)i] * s;
            err = std::max(err, std::fabs(marg[(size_t)i] / w[(size_t)i] - 1.0));
        }
        if (err < 3e-14) { conv = true; break; }
        for (int i = 0; i < n; ++i) v[(size_t)i] *= std::sqrt(w[(size_t)i] / marg[(size_t)i]);
    }
    if (!conv) return false;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) K[(size_t)i * n + j] = (v[(size_t)i] * J[(size_t)i * n + j] * v[(size_t)j]) / w[(size_t)i];
    return true;
}

// ---- variance-preserving rectified rates ---------------------------------------------------
// lam(u) = (s u - t)^+ / E_w[(s u - t)^+] with E_w lam = 1 and Var_w lam = var (s = sign of the
// loading); var = 0 or a threshold below every node gives the linear rate 1 + s sqrt(var) u.
struct VpTables {
    int n = 0;
    std::vector<double> A, B, C, rvb;   // reverse cumulative sums of w u, w, w u^2; rel. variance per segment
};

bool vp_tables(const std::vector<double>& u, const std::vector<double>& w, VpTables& T) {
    const int n = (int)u.size();
    T.n = n;
    T.A.assign((size_t)n, 0.0); T.B.assign((size_t)n, 0.0); T.C.assign((size_t)n, 0.0);
    double a = 0, b = 0, c = 0;
    for (int i = n - 1; i >= 0; --i) {
        a += w[(size_t)i] * u[(size_t)i]; b += w[(size_t)i]; c += w[(size_t)i] * u[(size_t)i] * u[(size_t)i];
        T.A[(size_t)i] = a; T.B[(size_t)i] = b; T.C[(size_t)i] = c;
    }
    T.rvb.resize((size_t)n - 1);
    for (int j = 1; j < n; ++j) {
        const double tb = u[(size_t)j - 1];
        const double E1 = T.A[(size_t)j] - tb * T.B[(size_t)j];
        const double E2 = T.C[(size_t)j] - 2 * tb * T.A[(size_t)j] + tb * tb * T.B[(size_t)j];
        T.rvb[(size_t)j - 1] = E2 / (E1 * E1) - 1.0;
        if (j > 1 && !(T.rvb[(size_t)j - 1] > T.rvb[(size_t)j - 2])) return false;
    }
    return true;
}

// lam (n values) of one group; returns 1 (variance beyond the state cap), 2 (root outside its
// segment) or 0
int vp_rate(const VpTables& T, const std::vector<double>& u, const std::vector<double>& w, double v, double sgn,
            double* lam) {
    const int n = T.n;
    if (v >= T.rvb.back()) return 1;
    const int j = (int)(std::upper_bound(T.rvb.begin(), T.rvb.end(), v) - T.rvb.begin());
    const double s = sgn >= 0 ? 1.0 : -1.0;
    if (j == 0) {                                   // linear branch: exactly 1 + s sqrt(v) u
        const double sv = std::sqrt(v);
        for (int i = 0; i < n; ++i) lam[i] = 1.0 + sv * (s * u[(size_t)i]);
        return 0;
    }
    const double a = T.A[(size_t)j], b = T.B[(size_t)j], c = T.C[(size_t)j];
    const double q2 = b - (1 + v) * b * b, q1 = 2 * a * ((1 + v) * b - 1), q0 = c - (1 + v) * a * a;
    const double lo = u[(size_t)std::max(j - 1, 0)], hi = u[(size_t)j];
    const double disc = std::sqrt(std::max(q1 * q1 - 4 * q2 * q0, 0.0));
    const double r1 = q2 != 0 ? (-q1 - disc) / (2 * q2) : -q0 / q1;
    const double r2 = q2 != 0 ? (-q1 + disc) / (2 * q2) : -q0 / q1;
    const double t = (r1 >= lo && r1 < hi) ? r1 : r2;
    if (!(t >= lo - 1e-12 * (1 + std::fabs(lo)) && t <= hi)) return 2;
    double norm = 0.0;
    for (int i = 0; i < n; ++i) {
        const double xv = std::max(s * u[(size_t)i] - t, 0.0);
        lam[i] = xv;
        norm += xv * w[(size_t)i];
    }
    for (int i = 0; i < n; ++i) lam[i] /= norm;
    return 0;
}

// ---- chain variance of sum_s m_s(U_s) over the stationary chain ----------------------------
double chain_variance(const std::vector<std::vector<double>>& ms, const std::vector<double>& w,
                      const std::vector<double>& K) {
    const int n = (int)w.size();
    std::vector<double> h((size_t)n), hp((size_t)n), mu((size_t)n);
    double var = 0.0;
    for (size_t s = 0; s < ms.size(); ++s) {
        double mean = 0.0;
        for (int i = 0; i < n; ++i) mean += w[(size_t)i] * ms[s][(size_t)i];
        for (int i = 0; i < n; ++i) mu[(size_t)i] = ms[s][(size_t)i] - mean;
        double d = 0.0;
        for (int i = 0; i < n; ++i) d += w[(size_t)i] * (mu[(size_t)i] * mu[(size_t)i]);
        var += d;
        if (s == 0) {
            for (int i = 0; i < n; ++i) h[(size_t)i] = w[(size_t)i] * mu[(size_t)i];
        } else {
            const double* Ks = K.data() + (s - 1) * (size_t)n * n;
            for (int j = 0; j < n; ++j) {
                double acc = 0.0;
                for (int i = 0; i < n; ++i) acc += Ks[(size_t)i * n + j] * h[(size_t)i];
                hp[(size_t)j] = acc;
            }
            double e = 0.0;
            for (int i = 0; i < n; ++i) e += mu[(size_t)i] * hp[(size_t)i];
            var += 2 * e;
            for (int i = 0; i < n; ++i) h[(size_t)i] = hp[(size_t)i] + w[(size_t)i] * mu[(size_t)i];
        }
    }
    return var;
}

// ---- Brent's root finder (Brent 1973, ch. 4: inverse quadratic / secant steps guarded by bisection)
template <typename F>
double brent_root(F f, double xa, double xb, double xtol, double rtol, int maxiter, bool& ok) {
    double xpre = xa, xcur = xb, xblk = 0.0, fblk = 0.0, spre = 0.0, scur = 0.0;
    double fpre = f(xpre), fcur = f(xcur);
    ok = true;
    if (fpre == 0) return xpre;
    if (fcur == 0) return xcur;
    if ((fpre > 0) == (fcur > 0)) { ok = false; return xcur; }
    for (int i = 0; i < maxiter; ++i) {
        if (fpre != 0 && fcur != 0 && (std::signbit(fpre) != std::signbit(fcur))) {
            xblk = xpre; fblk = fpre;
            spre = scur = xcur - xpre;
        }
        if (std::fabs(fblk) < std::fabs(fcur)) {
            xpre = xcur; xcur = xblk; xblk = xpre;
            fpre = fcur; fcur = fblk; fblk = fpre;
        }
        const double delta = (xtol + rtol * std::fabs(xcur)) / 2;
        const double sbis = (xblk - xcur) / 2;
        if (fcur == 0 || std::fabs(sbis) < delta) return xcur;
        if (std::fabs(spre) > delta && std::fabs(fcur) < std::fabs(fpre)) {
            double stry;
            if (xpre == xblk) {
                stry = -fcur * (xcur - xpre) / (fcur - fpre);                    // secant
            } else {
                const double dpre = (fpre - fcur) / (xpre - xcur);
                const double dblk = (fblk - fcur) / (xblk - xcur);
                stry = -fcur * (fblk * dblk - fpre * dpre) / (dblk * dpre * (fblk - fpre));   // inverse quadratic
            }
            if (2 * std::fabs(stry) < std::min(std::fabs(spre), 3 * std::fabs(sbis) - delta)) {
                spre = scur; scur = stry;
            } else {
                spre = sbis; scur = sbis;
            }
        } else {
            spre = sbis; scur = sbis;
        }
        xpre = xcur; fpre = fcur;
        if (std::fabs(scur) > delta) xcur += scur;
        else xcur += (sbis > 0 ? delta : -delta);
        fcur = f(xcur);
    }
    ok = false;
    return xcur;
}

}  // namespace
}  // namespace sglh

extern "C" {

sgl_status sgl_vp_build(sgl_ctx* ctx, int nstate, int n_shells, const int64_t* shell_start, const double* W,
                        const double* kap, const double* gam, const double* phi, const double* rho, const double* fvar,
                        double target_kappa, double target_gamma, double eta_in, double* eta_out) {
    if (!ctx) return SGL_ERR_VALUE;
    if (nstate < 2 || nstate > 256 || n_shells < 1 || !shell_start || !rho && n_shells > 1 || !fvar)
        return fail(ctx, SGL_ERR_VALUE, "sgl_vp_build: invalid sizes or arrays");
    if (shell_start[0] != 0) return fail(ctx, SGL_ERR_VALUE, "sgl_vp_build: shell_start[0] must be 0");
    for (int s = 0; s < n_shells; ++s)
        if (shell_start[s + 1] < shell_start[s]) return fail(ctx, SGL_ERR_VALUE, "sgl_vp_build: shell_start not ascending");
    const long long nc = shell_start[n_shells];
    if (nc > 0 && (!W || !kap || !gam || !phi)) return fail(ctx, SGL_ERR_VALUE, "sgl_vp_build: cell arrays are NULL");
    for (long long c = 0; c < nc; ++c)
        if (!std::isfinite(W[c]) || !std::isfinite(kap[c]) || !std::isfinite(gam[c]) || !std::isfinite(phi[c]))
            return fail(ctx, SGL_ERR_VALUE, "sgl_vp_build: non-finite cell value");
    for (int s = 0; s + 1 < n_shells; ++s)
        if (!(std::fabs(rho[s]) < 1.0)) return fail(ctx, SGL_ERR_VALUE, "sgl_vp_build: |rho| must be < 1");
    HostTimer ht(ctx);
    const int n = nstate;
    // ---- latent states, transitions
    std::vector<double> u, w;
    hermegauss(n, u, w);
    std::vector<double> K((size_t)std::max(0, n_shells - 1) * n * n);
    std::atomic<int> bad_k{0};
    HostPool::get().run(std::max(0, n_shells - 1), [&](int s) {
        if (!transition(u, w, rho[s], K.data() + (size_t)s * n * n)) bad_k = 1;
    });
    if (bad_k) return fail(ctx, SGL_ERR_VALUE, "sgl_vp_build: stationary transition balancing did not converge");
    VpTables T;
    if (!vp_tables(u, w, T)) return fail(ctx, SGL_ERR_VALUE, "sgl_vp_build: state grid not usable for vp rates");
    // ---- per shell: unique loadings (groups), the group of each cell, sum_{c in g} W kap
    struct Shell { std::vector<double> ph, wk; std::vector<int> gidx; };
    std::vector<Shell> sh((size_t)n_shells);
    HostPool::get().run(n_shells, [&](int s) {
        const long long c0 = shell_start[s], c1 = shell_start[s + 1];
        Shell& S = sh[(size_t)s];
        std::vector<double> v(phi + c0, phi + c1);
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
        S.ph = v;
        S.gidx.resize((size_t)(c1 - c0));
        S.wk.assign(v.size(), 0.0);
        for (long long c = c0; c < c1; ++c) {
            const int g = (int)(std::lower_bound(v.begin(), v.end(), phi[c]) - v.begin());
            S.gidx[(size_t)(c - c0)] = g;
            S.wk[(size_t)g] += W[c] * kap[c];
        }
    });
    ht.lap("vp_groups");
    // ---- eta: the model's kappa clustering variance equals target_kappa
    std::atomic<int> rate_err{0};
    auto variance = [&](double eta) {
        std::vector<std::vector<double>> ms((size_t)n_shells, std::vector<double>((size_t)n, 0.0));
        HostPool::get().run(n_shells, [&](int s) {
            const Shell& S = sh[(size_t)s];
            std::vector<double> lam((size_t)n);
            std::vector<double>& m = ms[(size_t)s];
            for (size_t g = 0; g < S.ph.size(); ++g) {
                const double ph = S.ph[g];
                const int e = vp_rate(T, u, w, eta * fvar[s] * ph * ph, ph > 0 ? 1.0 : (ph < 0 ? -1.0 : 0.0), lam.data());
                if (e) { rate_err = e; return; }
                for (int i = 0; i < n; ++i) m[(size_t)i] += lam[(size_t)i] * S.wk[g];
            }
        });
        return chain_variance(ms, w, K);
    };
    double eta = eta_in;
    if (!(eta > 0)) {
        // brentq in ln eta; the bracket starts at [1/1.5, 1.5] and widens x1.5 per side until it
        // brackets, within [1e-3, 1e4] (Closure.calibrate)
        auto fun = [&](double le) { return variance(std::exp(le)) - target_kappa; };
        const double llo = std::log(1e-3), lhi = std::log(1e4);
        double a = -std::log(1.5), b = std::log(1.5);
        double fa = fun(a), fb = fun(b);
        while (fa * fb > 0 && !rate_err) {
            if (fa > 0 && a > llo) { b = a; fb = fa; a -= std::log(1.5); fa = fun(a); }
            else if (fb < 0 && b < lhi) { a = b; fa = fb; b += std::log(1.5); fb = fun(b); }
            else return fail(ctx, SGL_ERR_VALUE, "sgl_vp_build: kappa clustering target outside [1e-3, 1e4] in eta");
        }
        if (rate_err) return fail(ctx, SGL_ERR_VALUE, "sgl_vp_build: vp rate outside the state grid's range");
        bool ok = true;
        const double root = brent_root(fun, a, b, 2e-12, 4 * std::numeric_limits<double>::epsilon(), 100, ok);
        if (!ok || rate_err) return fail(ctx, SGL_ERR_VALUE, "sgl_vp_build: eta calibration did not converge");
        eta = std::exp(root);
    }
    ht.lap("vp_calibrate");
    // ---- unique (kap, gam) cells over all shells, lexicographic
    std::vector<long long> ord((size_t)nc);
    std::iota(ord.begin(), ord.end(), 0LL);
    std::sort(ord.begin(), ord.end(), [&](long long x, long long y) {
        return kap[x] < kap[y] || (kap[x] == kap[y] && (gam[x] < gam[y] || (gam[x] == gam[y] && x < y)));
    });
    std::vector<double> ku, gu;
    std::vector<int32_t> inv((size_t)nc);
    for (long long i = 0; i < nc; ++i) {
        const long long c = ord[(size_t)i];
        if (ku.empty() || kap[c] != ku.back() || gam[c] != gu.back()) { ku.push_back(kap[c]); gu.push_back(gam[c]); }
        inv[(size_t)c] = (int32_t)(ku.size() - 1);
    }
    // ---- per shell: cells ordered by group (stable), group offsets, rates and their intervals
    std::vector<long long> g_off((size_t)n_shells + 1, 0);
    for (int s = 0; s < n_shells; ++s) g_off[(size_t)s + 1] = g_off[(size_t)s] + (long long)sh[(size_t)s].ph.size();
    const long long ng = g_off[(size_t)n_shells];
    std::vector<int32_t> cu((size_t)nc), glo((size_t)ng), ghi((size_t)ng), sh_g((size_t)n_shells + 1);
    std::vector<double> cw((size_t)nc), ga((size_t)ng), gb((size_t)ng), gc((size_t)ng);
    std::vector<int64_t> gstart((size_t)ng + 1, 0);
    for (int s = 0; s <= n_shells; ++s) sh_g[(size_t)s] = (int32_t)g_off[(size_t)s];
    std::atomic<int> interval_err{0};
    HostPool::get().run(n_shells, [&](int s) {
        const Shell& S = sh[(size_t)s];
        const long long c0 = shell_start[s], ncs = shell_start[s + 1] - c0;
        const long long G = (long long)S.ph.size(), gbase = g_off[(size_t)s];
        std::vector<long long> cnt((size_t)G + 1, 0);
        for (long long i = 0; i < ncs; ++i) ++cnt[(size_t)S.gidx[(size_t)i] + 1];
        for (long long g = 0; g < G; ++g) cnt[(size_t)g + 1] += cnt[(size_t)g];
        for (long long g = 0; g < G; ++g) gstart[(size_t)(gbase + g)] = c0 + cnt[(size_t)g];
        std::vector<long long> fill(cnt.begin(), cnt.end() - 1);
        for (long long i = 0; i < ncs; ++i) {
            const long long dst = c0 + fill[(size_t)S.gidx[(size_t)i]]++;
            cu[(size_t)dst] = inv[(size_t)(c0 + i)];
            cw[(size_t)dst] = W[c0 + i];
        }
        std::vector<double> lam((size_t)n), d((size_t)n);
        for (long long g = 0; g < G; ++g) {
            const double ph = S.ph[(size_t)g];
            if (vp_rate(T, u, w, eta * fvar[s] * ph * ph, ph > 0 ? 1.0 : (ph < 0 ? -1.0 : 0.0), lam.data())) {
                interval_err = 1; return;
            }
            // rate_intervals: the rate D = lam - 1 is affine on one interval of active states
            int lo_i = -1, hi_i = -1, count = 0;
            for (int i = 0; i < n; ++i) {
                d[(size_t)i] = lam[(size_t)i] - 1.0;
                if (d[(size_t)i] + 1.0 > 0) { ++count; if (lo_i < 0) lo_i = i; hi_i = i; }
            }
            if (count == 0 || hi_i - lo_i + 1 != count) { interval_err = 2; return; }
            const bool all_active = count == n;
            const double c = all_active ? 0.0 : -1.0;
            const double first = all_active ? d[(size_t)lo_i] : d[(size_t)lo_i] + 1.0;
            const double last = all_active ? d[(size_t)hi_i] : d[(size_t)hi_i] + 1.0;
            const double span = u[(size_t)hi_i] - u[(size_t)lo_i];
            const double a = span != 0 ? (last - first) / span : 0.0;
            const double b = all_active ? 0.5 * (first + last - a * (u[(size_t)lo_i] + u[(size_t)hi_i]))
                                        : (a >= 0 ? first : last);
            const double anchor = all_active ? 0.0 : (a >= 0 ? u[(size_t)lo_i] : u[(size_t)hi_i]);
            if (!all_active && lo_i != 0 && hi_i != n - 1) { interval_err = 3; return; }
            for (int i = 0; i < n; ++i) {
                const bool act = d[(size_t)i] + 1.0 > 0;
                const double model = c + (act ? (u[(size_t)i] - anchor) * a + b : 0.0);
                if (std::fabs(model - d[(size_t)i]) / std::max(1.0, std::fabs(d[(size_t)i])) > 2e-12) { interval_err = 4; return; }
            }
            ga[(size_t)(gbase + g)] = a; gb[(size_t)(gbase + g)] = b; gc[(size_t)(gbase + g)] = c;
            glo[(size_t)(gbase + g)] = lo_i; ghi[(size_t)(gbase + g)] = hi_i;
        }
    });
    gstart[(size_t)ng] = nc;
    if (interval_err)
        return fail(ctx, SGL_ERR_VALUE, "sgl_vp_build: a group's vp rate is not affine on one interval of states (" +
                                            std::to_string(interval_err.load()) + ")");
    ht.lap("vp_cells");
    if (eta_out) *eta_out = eta;
    return sgl_vp_set(ctx, n, u.data(), w.data(), n_shells, K.data(), (int)ku.size(), ku.data(), gu.data(), nc,
                      cu.data(), cw.data(), (int)ng, gstart.data(), sh_g.data(), ga.data(), gb.data(), gc.data(),
                      glo.data(), ghi.data(), target_gamma);
}

}  // extern "C"
