/*
 * fwi_oracle.cpp -- CPU oracle for the FWI per-shot hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is built into oracle/_build/liboracle.so,
 * which is loaded only by tests/, by __graft_entry__.smoke() and by the
 * cpu_baseline / --impl reference legs of bench.py.  The product library
 * (fwi_gb300/csrc) never links, loads or calls it.
 *
 * It restates, in plain C++ templated on the real type (float = the
 * reference's default REAL, double = the FP64 error reference), the semantics
 * of the reference Fortran solver of ejimeneztejero/FWI:
 *
 *   src/solver_FD_coeffs.f90:1-73        fd_coef()
 *   src/solver_PML_coeffs.f90:1-75       pml_coeffs()
 *   src/solver_space_derivs.f90:1-131    deriv2x/deriv2y/derivx/derivy()
 *   src/solver_PML_matrices.f90:1-112    pml_strip_x/pml_strip_y/pml_corner()
 *   src/solver_acoustic_SS.f90:9-645     solver_acoustic_ss()
 *   src/Misfit.f90:1-77, Misfit_L2.f90   misfit_function()
 *   src/Beta_calculous.f90:1-25          beta_calculous()
 *   src/calculate_misfit_gradient.f90    time_rules(), gradient batch, mask
 *   src/get_mcs_data.f90:106-155,331-369,503-512   geometry, ricker
 *
 * Every floating-point expression is evaluated in the order the Fortran
 * source writes it (left to right, ** 2 as a product).  The file must be
 * compiled with -ffp-contract=off and without -ffast-math so that no
 * multiply-add is fused and nothing is reassociated.
 *
 * The structure deliberately keeps the reference's per-step passes (four
 * full-grid derivative arrays, separate strip arrays, copy-based time
 * rotation), so that timing it gives the reference's CPU cost.
 *
 * Pinning: tests/golden holds vectors produced by executing the reference's
 * own Fortran source (interpreted in FP32 by tests/golden/fortran_exec.py);
 * tests/test_oracle_golden.py checks this oracle against them bit for bit.
 */
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace {

/* Column-major 2-D array with 1-based accessors, the way the Fortran source
 * indexes it.  Element (i, j) lives at (i-1) + (j-1)*n1. */
template <typename R>
struct A2 {
    int n1 = 0, n2 = 0;
    std::vector<R> v;
    A2() = default;
    A2(int a, int b) : n1(a), n2(b), v((size_t)a * (size_t)b, R(0)) {}
    R& operator()(int i, int j) { return v[(size_t)(i - 1) + (size_t)(j - 1) * n1]; }
    const R& operator()(int i, int j) const { return v[(size_t)(i - 1) + (size_t)(j - 1) * n1]; }
    R* data() { return v.data(); }
    void zero() { std::fill(v.begin(), v.end(), R(0)); }
};

template <typename R> R r_exp(R x);
template <> float r_exp<float>(float x) { return expf(x); }
template <> double r_exp<double>(double x) { return exp(x); }
template <typename R> R r_log(R x);
template <> float r_log<float>(float x) { return logf(x); }
template <> double r_log<double>(double x) { return log(x); }
template <typename R> R r_sqrt(R x);
template <> float r_sqrt<float>(float x) { return sqrtf(x); }
template <> double r_sqrt<double>(double x) { return sqrt(x); }

/* finite_difference_coef (solver_FD_coeffs.f90:1-73).  coef has acc+1
 * entries; num=1 gives the first-derivative taps, num=2 the second-derivative
 * taps with the centre tap halved (:68). */
template <typename R>
void fd_coef(int num, int acc, R* coef) {
    for (int i = 0; i <= acc; ++i) coef[i] = R(0);
    if (num == 1) {
        if (acc == 1) { coef[0] = R(0); coef[1] = R(1 / 2); /* integer 1/2 == 0 */ }
        if (acc == 3) {
            coef[0] = R(0); coef[1] = R(3) / R(4); coef[2] = -(R(3) / R(20)); coef[3] = R(1) / R(60);
        }
        if (acc == 4) {
            coef[0] = R(0); coef[1] = R(4) / R(5); coef[2] = -(R(1) / R(5));
            coef[3] = R(4) / R(105); coef[4] = -(R(1) / R(280));
        }
        /* acc == 5: all zero (:29-36) */
    }
    if (num == 2) {
        if (acc == 3) {
            coef[0] = -(R(49) / R(18)); coef[1] = R(3) / R(2); coef[2] = -(R(3) / R(20)); coef[3] = R(1) / R(90);
        }
        if (acc == 4) {
            coef[0] = -(R(205) / R(72)); coef[1] = R(8) / R(5); coef[2] = -(R(1) / R(5));
            coef[3] = R(8) / R(315); coef[4] = -(R(1) / R(560));
        }
        if (acc == 5) {
            coef[0] = -(R(5269) / R(1800)); coef[1] = R(5) / R(3); coef[2] = -(R(5) / R(21));
            coef[3] = R(5) / R(126); coef[4] = -(R(5) / R(1008)); coef[5] = R(1) / R(3150);
        }
        coef[0] = coef[0] / R(2);
    }
}

/* PML_coeffs (solver_PML_coeffs.f90:1-75).  fA/fB have dn entries (1..acc
 * stay zero, as the caller zero-initialises them, solver_acoustic_SS.f90:155);
 * the corner matrices are dn x dn column-major. */
template <typename R>
void pml_coeffs(int acc, int dPML, R dt, R d, int dn, A2<R>& fAv, A2<R>& fBv,
                A2<R>& ldA, A2<R>& rdA, A2<R>& luA, A2<R>& ruA,
                A2<R>& ldB, A2<R>& rdB, A2<R>& luB, A2<R>& ruB) {
    const R pi = R(3.14159265);
    const R Refl = R(0.00001);
    const R wPML = R(dPML - 1) * d;
    std::vector<R> yPML(dn + 1, R(0)), alpha(dn + 1, R(0)), sigma(dn + 1, R(0));
    auto fA = [&](int i) -> R& { return fAv(i, 1); };
    auto fB = [&](int i) -> R& { return fBv(i, 1); };
    for (int i = 1 + acc; i <= dPML + acc; ++i) {
        yPML[i] = R(i - (acc + 1)) * d;
        alpha[i] = R(30) * pi * (R(1) - (yPML[i] / wPML));
        const R q = yPML[i] / wPML;
        sigma[i] = (-((R(6000) * r_log<R>(Refl)) / (R(2) * wPML))) * (q * q);
    }
    for (int i = 1 + acc; i <= dPML + acc; ++i) {
        fA(i) = r_exp<R>((-(sigma[i] + alpha[i])) * dt);
        fB(i) = ((fA(i) - R(1)) * sigma[i]) / (sigma[i] + alpha[i]);
    }
    for (int i = dPML + acc + 1; i <= dn; ++i) {
        fA(i) = fA(dPML + acc);
        fB(i) = fB(dPML + acc);
    }
    for (int i = 1; i <= dn; ++i)
        for (int j = 1; j <= i; ++j) { rdA(j, i) = fA(i); rdB(j, i) = fB(i); }
    for (int i = 1; i <= dn; ++i)
        for (int j = i + 1; j <= dn; ++j) { rdA(j, i) = rdA(i, j); rdB(j, i) = rdB(i, j); }
    for (int i = 1; i <= dn; ++i)
        for (int j = 1; j <= dn - i + 1; ++j) { ldA(j, i) = fA(dn - i + 1); ldB(j, i) = fB(dn - i + 1); }
    for (int ix = 1; ix <= dn - 1; ++ix) {
        const int j = 2 + (ix - 1);
        for (int i = dn - (ix - 1); i <= dn; ++i) { ldA(j, i) = fA(j); ldB(j, i) = fB(j); }
    }
    for (int j = 1; j <= dn; ++j)
        for (int i = 1; i <= dn; ++i) {
            luA(j, i) = ldA(dn - j + 1, i); luB(j, i) = ldB(dn - j + 1, i);
            ruA(j, i) = rdA(dn - j + 1, i); ruB(j, i) = rdB(dn - j + 1, i);
        }
}

/* space_deriv2x / space_deriv2y / space_derivx / space_derivy
 * (solver_space_derivs.f90:1-131): undivided central differences over
 * interior lines acc+1..n-acc; the first and last acc lines copy the nearest
 * computed line. */
template <typename R>
void deriv2x(int acc, const R* coef, A2<R>& p, A2<R>& out) {
    const int nyt = p.n1, nxt = p.n2, j1 = 1 + acc, j2 = nxt - acc;
    for (int j = j1; j <= j2; ++j)
        for (int r = 1; r <= nyt; ++r) {
            R s = R(0);
            for (int i = 1; i <= acc + 1; ++i) s = s + coef[i - 1] * (p(r, j + (i - 1)) + p(r, j - (i - 1)));
            out(r, j) = s;
        }
    for (int j = 1; j <= j1 - 1; ++j) for (int r = 1; r <= nyt; ++r) out(r, j) = out(r, acc + 1);
    for (int j = j2 + 1; j <= nxt; ++j) for (int r = 1; r <= nyt; ++r) out(r, j) = out(r, nxt - acc);
}
template <typename R>
void deriv2y(int acc, const R* coef, A2<R>& p, A2<R>& out) {
    const int nyt = p.n1, nxt = p.n2, j1 = 1 + acc, j2 = nyt - acc;
    for (int k = 1; k <= nxt; ++k)
        for (int j = j1; j <= j2; ++j) {
            R s = R(0);
            for (int i = 1; i <= acc + 1; ++i) s = s + (p(j + (i - 1), k) + p(j - (i - 1), k)) * coef[i - 1];
            out(j, k) = s;
        }
    for (int k = 1; k <= nxt; ++k) {
        for (int j = 1; j <= j1 - 1; ++j) out(j, k) = out(acc + 1, k);
        for (int j = j2 + 1; j <= nyt; ++j) out(j, k) = out(nyt - acc, k);
    }
}
template <typename R>
void derivx(int acc, const R* coef, A2<R>& p, A2<R>& out) {
    const int nyt = p.n1, nxt = p.n2, j1 = 1 + acc, j2 = nxt - acc;
    for (int j = j1; j <= j2; ++j)
        for (int k = 1; k <= nyt; ++k) {
            R s = R(0);
            for (int i = 1; i <= acc + 1; ++i) s = s + (p(k, j + (i - 1)) - p(k, j - (i - 1))) * coef[i - 1];
            out(k, j) = s;
        }
    for (int j = 1; j <= j1 - 1; ++j) for (int k = 1; k <= nyt; ++k) out(k, j) = out(k, acc + 1);
    for (int j = j2 + 1; j <= nxt; ++j) for (int k = 1; k <= nyt; ++k) out(k, j) = out(k, nxt - acc);
}
template <typename R>
void derivy(int acc, const R* coef, A2<R>& p, A2<R>& out) {
    const int nyt = p.n1, nxt = p.n2, j1 = 1 + acc, j2 = nyt - acc;
    for (int k = 1; k <= nxt; ++k)
        for (int j = j1; j <= j2; ++j) {
            R s = R(0);
            for (int i = 1; i <= acc + 1; ++i) s = s + (p(j + (i - 1), k) - p(j - (i - 1), k)) * coef[i - 1];
            out(j, k) = s;
        }
    for (int k = 1; k <= nxt; ++k) {
        for (int j = 1; j <= j1 - 1; ++j) out(j, k) = out(acc + 1, k);
        for (int j = j2 + 1; j <= nyt; ++j) out(j, k) = out(nyt - acc, k);
    }
}

/* One CPML region: a rectangular block of the padded grid starting at grid
 * row r0+1, column c0+1 (so strip element (j,i) is grid (r0+j, c0+i)), with
 * its own copies of the pressure and the memory variables, as the reference
 * keeps them (solver_acoustic_SS.f90:55-85). */
template <typename R>
struct Region {
    int r0, c0, nr, nc;
    A2<R> pm1, p0, p3;             /* *_pml_p_1, *_pml_p, *_pml_p_3 */
    A2<R> phx, phx1, chx, chx1;     /* x-direction phi/chi and their _1 copies */
    A2<R> phy, phy1, chy, chy1;     /* y-direction */
    Region(int r0_, int c0_, int nr_, int nc_)
        : r0(r0_), c0(c0_), nr(nr_), nc(nc_), pm1(nr_, nc_), p0(nr_, nc_), p3(nr_, nc_),
          phx(nr_, nc_), phx1(nr_, nc_), chx(nr_, nc_), chx1(nr_, nc_),
          phy(nr_, nc_), phy1(nr_, nc_), chy(nr_, nc_), chy1(nr_, nc_) {}
};

/* pml_matrices_x / _y / _xycorner (solver_PML_matrices.f90:1-112).
 * dir 0 = x, 1 = y.  factor(j,i) gives the A or B factor of strip element
 * (j,i).  deriv_phi is the strip-local first derivative of the current (i.e.
 * previous step's) phi along dir, clamped at both strip ends. */
template <typename R, typename FA, typename FB>
void pml_update(int dir, int acc, const R* coef1, Region<R>& g, A2<R>& deriv, A2<R>& deriv2,
                A2<R>& phi, A2<R>& phi_1, A2<R>& chi, A2<R>& chi_1, A2<R>& prop, FA fa, FB fb) {
    A2<R> dphi(g.nr, g.nc);
    if (dir == 0) derivx(acc, coef1, phi, dphi); else derivy(acc, coef1, phi, dphi);
    for (int i = 1; i <= g.nc; ++i)
        for (int j = 1; j <= g.nr; ++j) {
            const R A = fa(j, i), B = fb(j, i);
            phi(j, i) = A * phi_1(j, i) + B * deriv(g.r0 + j, g.c0 + i);
            chi(j, i) = A * chi_1(j, i) + B * (deriv2(g.r0 + j, g.c0 + i) + dphi(j, i));
        }
    for (int i = 1; i <= g.nc; ++i)
        for (int j = 1; j <= g.nr; ++j) prop(j, i) = dphi(j, i) + chi(j, i);
}

template <typename R>
struct SolverArgs {
    int iprop, NumSou, NumRec;
    const int *nxSou, *nySou, *nxRec, *nyRec;
    const R *S, *Sadj;
    R d, dt;
    int ny, nx;
    const R* ctmp;
    int store_snap, nt_Store, nt;
    R* kernel;
    R* Fields;
    R* Rec_point;
    int acc, dPML;
};

/* solver_acoustic_SS (solver_acoustic_SS.f90:9-645) with free_surface = 1. */
template <typename R>
void solver_acoustic_ss(const SolverArgs<R>& a) {
    const int acc = a.acc, dPML = a.dPML, ny = a.ny, nx = a.nx, nt = a.nt;
    const int dn = dPML + 2 * acc;                       /* :99 */
    const int nxt = nx + 2 * dn, nyt = dn + ny + dn;     /* :120-121 */
    const int NumRec = a.NumRec, NumSou = a.NumSou;

    for (size_t i = 0; i < (size_t)nt * NumRec; ++i) a.Rec_point[i] = R(0);   /* :92 */

    std::vector<int> nxs, nys, nxreco(NumRec), nyreco(NumRec);
    if (a.iprop != 2) {
        nxs.resize(NumSou); nys.resize(NumSou);
        for (int j = 0; j < NumSou; ++j) { nxs[j] = dn + a.nxSou[j]; nys[j] = dn + a.nySou[j]; }
        for (int j = 0; j < NumRec; ++j) { nxreco[j] = dn + a.nxRec[j]; nyreco[j] = dn + a.nyRec[j]; }
    } else {
        nxs.resize(NumRec); nys.resize(NumRec);
        for (int j = 0; j < NumRec; ++j) { nxs[j] = dn + a.nxRec[j]; nys[j] = dn + a.nyRec[j]; }
    }

    A2<R> source(nyt, nxt), p_1(nyt, nxt), p(nyt, nxt), p_3(nyt, nxt), c(nyt, nxt), c2(nyt, nxt);
    A2<R> d2x(nyt, nxt), d2y(nyt, nxt), dx(nyt, nxt), dy(nyt, nxt);
    A2<R> ctmp(ny, nx);
    std::copy(a.ctmp, a.ctmp + (size_t)ny * nx, ctmp.v.begin());

    /* velocity extension into the pads (:271-290) */
    for (int i = 1; i <= nx; ++i) for (int j = 1; j <= ny; ++j) c(dn + j, dn + i) = ctmp(j, i);
    for (int i = 1; i <= dn; ++i) {
        for (int k = 1; k <= nx; ++k) c(i, dn + k) = ctmp(1, k);
        for (int j = 1; j <= dn; ++j) { c(i, j) = ctmp(1, 1); c(i, dn + nx + j) = ctmp(1, nx); }
    }
    for (int i = dn + ny + 1; i <= dn + ny + dn; ++i) {
        for (int k = 1; k <= nx; ++k) c(i, dn + k) = ctmp(ny, k);
        for (int j = 1; j <= dn; ++j) { c(i, j) = ctmp(ny, 1); c(i, dn + nx + j) = ctmp(ny, nx); }
    }
    for (int i = 1; i <= dn; ++i)
        for (int j = 1; j <= ny; ++j) { c(dn + j, i) = ctmp(j, 1); c(dn + j, dn + nx + i) = ctmp(j, nx); }
    {
        const R dt2 = a.dt * a.dt, d2 = a.d * a.d;   /* c**2*dt**2/d**2 (:292) */
        for (size_t i = 0; i < c.v.size(); ++i) c2.v[i] = ((c.v[i] * c.v[i]) * dt2) / d2;
    }

    A2<R> fA(dn, 1), fB(dn, 1), ldA(dn, dn), rdA(dn, dn), luA(dn, dn), ruA(dn, dn);
    A2<R> ldB(dn, dn), rdB(dn, dn), luB(dn, dn), ruB(dn, dn);
    pml_coeffs<R>(acc, dPML, a.dt, a.d, dn, fA, fB, ldA, rdA, luA, ruA, ldB, rdB, luB, ruB);

    std::vector<R> coef1(acc + 1), coef2(acc + 1);
    fd_coef<R>(1, acc, coef1.data());
    fd_coef<R>(2, acc, coef2.data());

    /* regions (grid offsets r0,c0 are the 0-based start) */
    Region<R> xr(dn, dn + nx, ny, dn), xl(dn, 0, ny, dn), yd(dn + ny, dn, dn, nx);
    Region<R> ld(dn + ny, 0, dn, dn), rd(dn + ny, dn + nx, dn, dn);
    Region<R> yu(0, dn, dn, nx), lu(0, 0, dn, dn), ru(0, dn + nx, dn, dn);
    A2<R> x_prop(ny, dn), y_prop(dn, nx), corner_prop(dn, dn);

    int l = 1, snap = (a.iprop == 1) ? 0 : (a.iprop == 2 ? a.nt_Store : 0);
    const R half = R(0.5);

    auto strip_p3 = [&](Region<R>& g, A2<R>& prop) {
        for (int i = 1; i <= g.nc; ++i)
            for (int j = 1; j <= g.nr; ++j) {
                const int gy = g.r0 + j, gx = g.c0 + i;
                g.p3(j, i) = ((-g.pm1(j, i)) + R(2) * g.p0(j, i)) +
                             c2(gy, gx) * ((d2x(gy, gx) + d2y(gy, gx)) + prop(j, i));
            }
    };
    auto corner_add = [&](Region<R>& g, A2<R>& prop) {
        for (int i = 1; i <= g.nc; ++i)
            for (int j = 1; j <= g.nr; ++j) g.p3(j, i) = g.p3(j, i) + c2(g.r0 + j, g.c0 + i) * prop(j, i);
    };
    auto rotate = [&](Region<R>& g) {
        g.pm1.v = g.p0.v; g.p0.v = g.p3.v;
        g.phx1.v = g.phx.v; g.chx1.v = g.chx.v; g.phy1.v = g.phy.v; g.chy1.v = g.chy.v;
    };
    auto writeback = [&](Region<R>& g) {
        for (int i = 1; i <= g.nc; ++i)
            for (int j = 1; j <= g.nr; ++j) p_3(g.r0 + j, g.c0 + i) = g.p3(j, i);
    };

    for (int k = 2; k <= nt; ++k) {
        l = l + 1;
        if (a.iprop != 2)
            for (int j = 0; j < NumSou; ++j) source(nys[j], nxs[j]) = a.S[(size_t)(k - 2) + (size_t)j * nt];
        if (a.iprop == 2)
            for (int j = 0; j < NumRec; ++j) source(nys[j], nxs[j]) = a.Sadj[(size_t)(k - 2) + (size_t)j * nt];

        deriv2x(acc, coef2.data(), p, d2x);
        deriv2y(acc, coef2.data(), p, d2y);
        derivx(acc, coef1.data(), p, dx);
        derivy(acc, coef1.data(), p, dy);

        /* x strips (:347-355): right uses factor(i), left factor(dn-i+1) */
        pml_update(0, acc, coef1.data(), xr, dx, d2x, xr.phx, xr.phx1, xr.chx, xr.chx1, x_prop,
                   [&](int, int i) { return fA(i, 1); }, [&](int, int i) { return fB(i, 1); });
        strip_p3(xr, x_prop);
        pml_update(0, acc, coef1.data(), xl, dx, d2x, xl.phx, xl.phx1, xl.chx, xl.chx1, x_prop,
                   [&](int, int i) { return fA(dn - i + 1, 1); }, [&](int, int i) { return fB(dn - i + 1, 1); });
        strip_p3(xl, x_prop);
        /* bottom strip (:359-362): factor(j) */
        pml_update(1, acc, coef1.data(), yd, dy, d2y, yd.phy, yd.phy1, yd.chy, yd.chy1, y_prop,
                   [&](int j, int) { return fA(j, 1); }, [&](int j, int) { return fB(j, 1); });
        strip_p3(yd, y_prop);
        /* bottom corners, x stage then y stage (:395-411) */
        pml_update(0, acc, coef1.data(), ld, dx, d2x, ld.phx, ld.phx1, ld.chx, ld.chx1, corner_prop,
                   [&](int j, int i) { return ldA(j, i); }, [&](int j, int i) { return ldB(j, i); });
        strip_p3(ld, corner_prop);
        pml_update(1, acc, coef1.data(), ld, dy, d2y, ld.phy, ld.phy1, ld.chy, ld.chy1, corner_prop,
                   [&](int j, int i) { return ldA(j, i); }, [&](int j, int i) { return ldB(j, i); });
        corner_add(ld, corner_prop);
        pml_update(0, acc, coef1.data(), rd, dx, d2x, rd.phx, rd.phx1, rd.chx, rd.chx1, corner_prop,
                   [&](int j, int i) { return rdA(j, i); }, [&](int j, int i) { return rdB(j, i); });
        strip_p3(rd, corner_prop);
        pml_update(1, acc, coef1.data(), rd, dy, d2y, rd.phy, rd.phy1, rd.chy, rd.chy1, corner_prop,
                   [&](int j, int i) { return rdA(j, i); }, [&](int j, int i) { return rdB(j, i); });
        corner_add(rd, corner_prop);

        /* free surface (:416-429) */
        for (int i = 1; i <= nxt; ++i) p_3(1 + dn, i) = R(0);
        for (int j = 1; j <= dn; ++j) {
            for (int i = 1; i <= nx; ++i) yu.p3(j, i) = p_3(dn + 1 + (1 - j), dn + i);
            for (int i = 1; i <= dn; ++i) {
                lu.p3(j, i) = p_3(dn + 1 + (1 - j), i);
                ru.p3(j, i) = p_3(dn + 1 + (1 - j), dn + nx + i);
            }
        }

        /* interior (:433-434) */
        for (int i = dn + 1; i <= dn + nx; ++i)
            for (int j = dn + 1; j <= dn + ny; ++j)
                p_3(j, i) = ((-p_1(j, i)) + R(2) * p(j, i)) + ((d2x(j, i) + d2y(j, i)) + source(j, i)) * c2(j, i);

        /* snapshot store (:438-454) / imaging condition (:457-473) */
        if (a.iprop == 1 && l == a.store_snap) {
            snap = snap + 1;
            for (int i = 1; i <= nx; ++i)
                for (int j = 1; j <= ny; ++j)
                    a.Fields[(size_t)(j - 1) + ((size_t)snap * nx + i - 1) * ny] =
                        ((p_3(dn + j, dn + i) - p_1(dn + j, dn + i)) * half) / a.dt;
            l = 0;
        }
        if (a.iprop == 2 && l == a.store_snap) {
            snap = snap - 1;
            const R ss = R(a.store_snap);
            for (int i = 1; i <= nx; ++i)
                for (int j = 1; j <= ny; ++j) {
                    const R F = a.Fields[(size_t)(j - 1) + ((size_t)snap * nx + i - 1) * ny];
                    const R k2 = -(((half * (p_3(dn + j, dn + i) - p_1(dn + j, dn + i))) * F) * ss);
                    R& K = a.kernel[(size_t)(j - 1) + (size_t)(i - 1) * ny];
                    K = K + k2;
                }
            l = 0;
        }

        /* strip write-back (:477-486) */
        writeback(yu); writeback(lu); writeback(ru);
        writeback(yd); writeback(ld); writeback(rd);
        writeback(xl); writeback(xr);

        /* time rotation (:491-547) */
        p_1.v = p.v;
        p.v = p_3.v;
        rotate(yu); rotate(yd); rotate(xl); rotate(xr); rotate(lu); rotate(ru); rotate(ld); rotate(rd);

        if (a.iprop != 2)
            for (int i = 0; i < NumRec; ++i)
                a.Rec_point[(size_t)(k - 2) + (size_t)i * nt] = p_3(nyreco[i], nxreco[i]);
    }
    if (nt >= 2)
        for (int i = 0; i < NumRec; ++i)
            a.Rec_point[(size_t)(nt - 1) + (size_t)i * nt] = a.Rec_point[(size_t)(nt - 2) + (size_t)i * nt];
}

/* Misfit_function + Misfit_L2 (Misfit.f90:1-77, Misfit_L2.f90:1-18,
 * is_not_cero auxiliar.f90:282-299), misfit_type = 1.  Returns the misfit
 * accumulated as the reference does (sequential, in R) in *mis_r and, for the
 * FP64 form, the same FP32/R terms 0.5*dt*r*r accumulated in double. */
template <typename R>
void misfit_function(int NumRec, int nt, R dt, const R* synth, const R* trace, R* mis_r, double* mis64, R* adj) {
    std::vector<R> S((size_t)nt * NumRec, R(0)), T((size_t)nt * NumRec, R(0));
    for (int j = 0; j < NumRec; ++j) {
        const R* tr = trace + (size_t)j * nt;
        const R* sy = synth + (size_t)j * nt;
        bool nz = false;
        for (int i = 0; i < nt; ++i) if (tr[i] != R(0)) { nz = true; break; }
        if (!nz) continue;
        R maxS = R(0), maxT = R(0);
        for (int i = 0; i < nt; ++i) { maxS = std::max(maxS, std::fabs(sy[i])); maxT = std::max(maxT, std::fabs(tr[i])); }
        if (maxS != R(0) && maxT != R(0))
            for (int i = 0; i < nt; ++i) { S[(size_t)j * nt + i] = sy[i] / maxS; T[(size_t)j * nt + i] = tr[i] / maxT; }
    }
    R m = R(0);
    double m64 = 0.0;
    const R hdt = R(0.5) * dt;
    for (int j = 0; j < NumRec; ++j)
        for (int k = 1; k <= nt; ++k) {
            const R r = S[(size_t)j * nt + k - 1] - T[(size_t)j * nt + k - 1];
            m = m + hdt * (r * r);
            m64 += 0.5 * (double)dt * (double)r * (double)r;
            const R rr = S[(size_t)j * nt + (nt - k)] - T[(size_t)j * nt + (nt - k)];
            adj[(size_t)j * nt + k - 1] = -rr;
        }
    *mis_r = m;
    *mis64 = m64;
}

}  // namespace

extern "C" {

int oracle_version(void) { return 1; }

void oracle_fd_coef_f32(int num, int acc, float* coef) { fd_coef<float>(num, acc, coef); }

/* fA, fB: dn floats; corners dn*dn column-major in the order ld, rd, lu, ru. */
void oracle_pml_coeffs_f32(int acc, int dPML, float dt, float d, float* fA, float* fB, float* cornA, float* cornB) {
    const int dn = dPML + 2 * acc;
    A2<float> a(dn, 1), b(dn, 1), ldA(dn, dn), rdA(dn, dn), luA(dn, dn), ruA(dn, dn), ldB(dn, dn), rdB(dn, dn),
        luB(dn, dn), ruB(dn, dn);
    pml_coeffs<float>(acc, dPML, dt, d, dn, a, b, ldA, rdA, luA, ruA, ldB, rdB, luB, ruB);
    std::copy(a.v.begin(), a.v.end(), fA);
    std::copy(b.v.begin(), b.v.end(), fB);
    const size_t n2 = (size_t)dn * dn;
    A2<float>* As[4] = {&ldA, &rdA, &luA, &ruA};
    A2<float>* Bs[4] = {&ldB, &rdB, &luB, &ruB};
    for (int q = 0; q < 4; ++q) {
        std::copy(As[q]->v.begin(), As[q]->v.end(), cornA + q * n2);
        std::copy(Bs[q]->v.begin(), Bs[q]->v.end(), cornB + q * n2);
    }
}

/* solver_acoustic_SS in FP32, Fortran layouts: S(nt,NumSou), Sadj(nt,NumRec),
 * ctmp(ny,nx), kernel(ny,nx), Fields(ny,nx*(nt_Store+1)), Rec_point(nt,NumRec). */
int oracle_solver_acoustic_ss_f32(int iprop, int NumSou, int NumRec, const int* nxSou, const int* nySou,
                                  const int* nxRec, const int* nyRec, const float* S, const float* Sadj, float d,
                                  float dt, int ny, int nx, const float* ctmp, int store_snap, int nt_Store, int nt,
                                  float* kernel, float* Fields, float* Rec_point, int acc, int dPML) {
    SolverArgs<float> a{iprop, NumSou, NumRec, nxSou, nySou, nxRec, nyRec, S, Sadj, d, dt, ny, nx, ctmp,
                        store_snap, nt_Store, nt, kernel, Fields, Rec_point, acc, dPML};
    solver_acoustic_ss<float>(a);
    return 0;
}

/* The same solver with every quantity in FP64 (the FP64 error reference). */
int oracle_solver_acoustic_ss_f64(int iprop, int NumSou, int NumRec, const int* nxSou, const int* nySou,
                                  const int* nxRec, const int* nyRec, const double* S, const double* Sadj, double d,
                                  double dt, int ny, int nx, const double* ctmp, int store_snap, int nt_Store, int nt,
                                  double* kernel, double* Fields, double* Rec_point, int acc, int dPML) {
    SolverArgs<double> a{iprop, NumSou, NumRec, nxSou, nySou, nxRec, nyRec, S, Sadj, d, dt, ny, nx, ctmp,
                         store_snap, nt_Store, nt, kernel, Fields, Rec_point, acc, dPML};
    solver_acoustic_ss<double>(a);
    return 0;
}

void oracle_misfit_function_f32(int NumRec, int nt, float dt, const float* synth, const float* trace,
                                float* misfit32, double* misfit64, float* adj) {
    misfit_function<float>(NumRec, nt, dt, synth, trace, misfit32, misfit64, adj);
}
void oracle_misfit_function_f64(int NumRec, int nt, double dt, const double* synth, const double* trace,
                                double* misfit, double* misfit64, double* adj) {
    misfit_function<double>(NumRec, nt, dt, synth, trace, misfit, misfit64, adj);
}

/* Beta_calculous (Beta_calculous.f90:1-25): Polak-Ribiere beta accumulated row
 * by row in FP32 like the reference, plus the same sums in FP64. */
void oracle_beta_calculous(const float* grad, const float* old, int nx, int ny, float* beta32, double* num64,
                           double* den64) {
    float Num = 0.f, Den = 0.f;
    double n64 = 0.0, d64 = 0.0;
    for (int i = 0; i < ny; ++i) {
        float dn_ = 0.f, dd_ = 0.f;
        for (int k = 0; k < nx; ++k) {
            const float v = grad[(size_t)i + (size_t)k * ny], vo = old[(size_t)i + (size_t)k * ny];
            dn_ = dn_ + v * (v - vo);
            dd_ = dd_ + vo * vo;
            n64 += (double)v * ((double)v - (double)vo);
            d64 += (double)vo * (double)vo;
        }
        Num = Num + dn_;
        Den = Den + dd_;
    }
    *beta32 = Num / Den;
    *num64 = n64;
    *den64 = d64;
}

/* Ricker_mcs (get_mcs_data.f90:331-369). */
void oracle_ricker(float freq, float dt, int nt, float* out) {
    const float pi = 3.14159265f, f0 = freq, t0 = 1.5f / f0, tmp = 10.f / f0;
    for (int i = 1; i <= nt; ++i) {
        const float t = (float)(i - 1) * dt;
        const float a = (pi * f0) * (t - t0);
        float s = (1.f - 2.f * (a * a)) * expf(-(1.f * (a * a)));
        if (t >= tmp) s = 0.f;
        out[i - 1] = s;
    }
}

/* MCS geometry (get_mcs_data.f90:113-114, 147-155, 503-512) for one shot
 * with the offset_header = 0 rule. */
void oracle_mcs_geometry(float xs, float shot_depth, float streamer_depth, float near_offset, float drec,
                         float dmodel, int NumRec, int* nxSou, int* nySou, int* nxRec, int* nyRec) {
    const float added_space_model = 0.f;
    const float pos_shot = added_space_model + std::fabs(xs);
    *nxSou = 1 + (int)std::ceil(pos_shot / dmodel);
    *nySou = 1 + (int)std::ceil(shot_depth / dmodel);
    for (int irec = 1; irec <= NumRec; ++irec) {
        const float pos_rec = (pos_shot - near_offset) - (float)(irec - 1) * drec;
        nxRec[irec - 1] = 1 + (int)std::ceil(pos_rec / dmodel);
        nyRec[irec - 1] = 1 + (int)std::ceil(streamer_depth / dmodel);
    }
}

/* Time rules of calculate_misfit_gradient.f90:198-203 (rho = 1000). */
void oracle_time_rules(const float* lambda, size_t n, float dmodel, float tfin, int store_snap, float* dt,
                       int* nt, int* nt_Store) {
    float mx = -INFINITY;
    for (size_t i = 0; i < n; ++i) mx = std::max(mx, lambda[i] / 1000.f);
    *dt = (dmodel / sqrtf(mx)) / 2.f;
    int ntt = 1 + (int)std::ceil(tfin / *dt);
    const float temp = (float)(ntt / store_snap);
    *nt_Store = (int)std::ceil(temp);
    *nt = *nt_Store * store_snap;
}

}  // extern "C"

namespace {
/* Round to the nearest bfloat16 (ties to even), returned as a float; finite inputs. */
float to_bf16(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);
    u &= 0xFFFF0000u;
    float y;
    std::memcpy(&y, &u, 4);
    return y;
}
float to_f16(float x) { return (float)(_Float16)x; }

/* Stored-snapshot forms, applied to Fields(ny, nx*(nt_Store+1)) between the
 * forward and the adjoint run (the imaging reads the stored values back):
 *   0 FP32 (the reference);
 *   1 / 2 FP16 / BF16 with one max-abs scale per snapshot: q = r(F * (2^14/m)),
 *     read back as q * (m/2^14), m = max|F| over the snapshot;
 *   3 / 4 FP16 / BF16 with a power-of-two scale per 128-column segment of a
 *     row: q = r(F * 2^(14-e)), read back exactly, 2^(e-1) <= the segment's
 *     max|F| < 2^e. */
void quantize_snapshots(float* F, int ny, int nx, int nsnap, int form) {
    if (form == 0) return;
    float (*rnd)(float) = (form == 1 || form == 3) ? to_f16 : to_bf16;
    for (int k = 0; k < nsnap; ++k) {
        float* A = F + (size_t)k * nx * ny;  // A[j + i*ny]
        if (form <= 2) {
            float m = 0.f;
            for (size_t c = 0; c < (size_t)nx * ny; ++c) m = std::max(m, std::fabs(A[c]));
            if (m == 0.f) continue;
            const float up = 16384.f / m, down = m / 16384.f;
            for (size_t c = 0; c < (size_t)nx * ny; ++c) A[c] = rnd(A[c] * up) * down;
        } else {
            for (int j = 0; j < ny; ++j)
                for (int i0 = 0; i0 < nx; i0 += 128) {
                    const int i1 = std::min(nx, i0 + 128);
                    float m = 0.f;
                    for (int i = i0; i < i1; ++i) m = std::max(m, std::fabs(A[j + (size_t)i * ny]));
                    int ex = 0;
                    if (m > 0.f) std::frexp(m, &ex);
                    const int sh = 14 - ex;
                    for (int i = i0; i < i1; ++i) {
                        float& v = A[j + (size_t)i * ny];
                        v = std::ldexp(rnd(std::ldexp(v, sh)), -sh);
                    }
                }
        }
    }
}
void quantize_snapshots(double*, int, int, int, int) {}

/* One shot of calculate_misfit_gradient (:236-323) with numtasks = 1 in R:
 * forward, misfit, adjoint.  kernel_out gets the shot's Grad_thread. */
template <typename R>
void shot_gradient(int ny, int nx, R d, R dt, int nt, int store_snap, int acc, int dPML, const R* vp,
                          int NumSou, const int* nxS, const int* nyS, const R* S, int NumRec, const int* nxR,
                          const int* nyR, const R* obs, int step, R* synth, R* kernel_out, R* mis_r, double* mis64,
                          int snap_form = 0) {
    const int nt_Store = nt / store_snap;
    std::vector<R> Fields((size_t)ny * nx * (nt_Store + 1), R(0));
    std::vector<R> adj((size_t)nt * NumRec, R(0)), dummy(1, R(0));
    SolverArgs<R> f{1, NumSou, NumRec, nxS, nyS, nxR, nyR, S, adj.data(), d, dt, ny, nx, vp,
                    store_snap, nt_Store, nt, kernel_out, Fields.data(), synth, acc, dPML};
    solver_acoustic_ss<R>(f);
    misfit_function<R>(NumRec, nt, dt, synth, obs, mis_r, mis64, adj.data());
    if (step != 1) return;
    quantize_snapshots(Fields.data(), ny, nx, nt_Store + 1, snap_form);
    std::fill(kernel_out, kernel_out + (size_t)ny * nx, R(0));
    std::vector<R> rec2((size_t)nt * NumRec, R(0));
    SolverArgs<R> b{2, NumSou, NumRec, nxS, nyS, nxR, nyR, S, adj.data(), d, dt, ny, nx, vp,
                    store_snap, nt_Store, nt, kernel_out, Fields.data(), rec2.data(), acc, dPML};
    solver_acoustic_ss<R>(b);
}

/* Batched gradient over shots, all in FP32 (or FP64 with _f64), each shot on
 * its own thread (nthreads at a time), like mpirun -np nthreads with one shot
 * per rank.  Per shot s: window x0[s] (0-based first model column), width
 * nxw[s]; sources/receivers are window-relative 1-based grid indices packed
 * shot after shot (offsets sou_off/rec_off, counts nsou/nrec); S and obs are
 * (nt, n) column-major blocks packed the same way.  Output: per-shot
 * kernels (ny x nxw[s], packed at kern_off[s]), per-shot misfits. */
template <typename R>
int gradient_batch(int nshots, int ny, R d, R dt, int nt, int store_snap, int acc, int dPML, const R* vp_model,
                          int nx_model, const int* x0, const int* nxw, const int* nsou, const int* sou_off,
                          const int* nxS, const int* nyS, const R* S, const int* nrec, const int* rec_off,
                          const int* nxR, const int* nyR, const R* obs, int step, const size_t* kern_off, R* kernels,
                          R* synth_all, R* mis_r, double* mis64, int nthreads, int snap_form = 0) {
    std::atomic<int> next{0};
    auto worker = [&]() {
        for (;;) {
            const int s = next.fetch_add(1);
            if (s >= nshots) break;
            const int nx = nxw[s];
            std::vector<R> vp((size_t)ny * nx);
            for (int i = 0; i < nx; ++i)
                for (int j = 0; j < ny; ++j) vp[(size_t)j + (size_t)i * ny] = vp_model[(size_t)j + (size_t)(x0[s] + i) * ny];
            std::vector<R> synth_local;
            R* synth = synth_all ? synth_all + (size_t)rec_off[s] * nt : nullptr;
            if (!synth) { synth_local.assign((size_t)nt * nrec[s], R(0)); synth = synth_local.data(); }
            shot_gradient<R>(ny, nx, d, dt, nt, store_snap, acc, dPML, vp.data(), nsou[s], nxS + sou_off[s],
                             nyS + sou_off[s], S + (size_t)sou_off[s] * nt, nrec[s], nxR + rec_off[s], nyR + rec_off[s],
                             obs + (size_t)rec_off[s] * nt, step, synth, kernels + kern_off[s], mis_r + s, mis64 + s,
                             snap_form);
        }
    };
    if (nthreads <= 1) { worker(); return 0; }
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; ++t) th.emplace_back(worker);
    for (auto& t : th) t.join();
    (void)nx_model;
    return 0;
}

}  // namespace

extern "C" {

int oracle_gradient_batch_f32(int nshots, int ny, float d, float dt, int nt, int store_snap, int acc, int dPML,
                              const float* vp_model, int nx_model, const int* x0, const int* nxw, const int* nsou,
                              const int* sou_off, const int* nxS, const int* nyS, const float* S, const int* nrec,
                              const int* rec_off, const int* nxR, const int* nyR, const float* obs, int step,
                              const size_t* kern_off, float* kernels, float* synth_all, float* mis32, double* mis64,
                              int nthreads) {
    return gradient_batch<float>(nshots, ny, d, dt, nt, store_snap, acc, dPML, vp_model, nx_model, x0, nxw, nsou,
                                 sou_off, nxS, nyS, S, nrec, rec_off, nxR, nyR, obs, step, kern_off, kernels,
                                 synth_all, mis32, mis64, nthreads);
}
/* quantize_snapshots on an array of nsnap snapshots (ny, nx) each, in place. */
void oracle_quantize_snapshots(float* F, int ny, int nx, int nsnap, int form) {
    quantize_snapshots(F, ny, nx, nsnap, form);
}

/* oracle_gradient_batch_f32 with the stored snapshots in the form snap_form
 * (quantize_snapshots): the precision forms' error against FP64. */
int oracle_gradient_batch_f32_form(int nshots, int ny, float d, float dt, int nt, int store_snap, int acc, int dPML,
                                   const float* vp_model, int nx_model, const int* x0, const int* nxw,
                                   const int* nsou, const int* sou_off, const int* nxS, const int* nyS, const float* S,
                                   const int* nrec, const int* rec_off, const int* nxR, const int* nyR,
                                   const float* obs, int step, const size_t* kern_off, float* kernels,
                                   float* synth_all, float* mis32, double* mis64, int nthreads, int snap_form) {
    return gradient_batch<float>(nshots, ny, d, dt, nt, store_snap, acc, dPML, vp_model, nx_model, x0, nxw, nsou,
                                 sou_off, nxS, nyS, S, nrec, rec_off, nxR, nyR, obs, step, kern_off, kernels,
                                 synth_all, mis32, mis64, nthreads, snap_form);
}
int oracle_gradient_batch_f64(int nshots, int ny, double d, double dt, int nt, int store_snap, int acc, int dPML,
                              const double* vp_model, int nx_model, const int* x0, const int* nxw, const int* nsou,
                              const int* sou_off, const int* nxS, const int* nyS, const double* S, const int* nrec,
                              const int* rec_off, const int* nxR, const int* nyR, const double* obs, int step,
                              const size_t* kern_off, double* kernels, double* synth_all, double* misr,
                              double* mis64, int nthreads) {
    return gradient_batch<double>(nshots, ny, d, dt, nt, store_snap, acc, dPML, vp_model, nx_model, x0, nxw, nsou,
                                  sou_off, nxS, nyS, S, nrec, rec_off, nxR, nyR, obs, step, kern_off, kernels,
                                  synth_all, misr, mis64, nthreads);
}

}  // extern "C"
