// FP64 CPU restatement of the reference time step -- TEST INFRASTRUCTURE ONLY
// (see lbm_oracle.h).  Every function cites the reference code it restates.
#include "lbm_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "shim/interpolation.h" // the ALGLIB bicubic spline restatement
// the boundary-type tables (identical numbers to include/system_files/*.txt)
#include "reference_tables.h"

namespace
{
const int NC = 9;
const int EX[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
const int EY[9] = {0, 0, 1, 0, -1, 1, 1, -1, -1};
const int OPPO[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};
const double W[9] = {4.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 9.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0, 1.0 / 36.0};
const double WF[9] = {0.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 3.0, 1.0 / 12.0, 1.0 / 12.0, 1.0 / 12.0, 1.0 / 12.0};
const double CS2 = 1. / 3.;
const double F1 = 3.0, F2 = 4.5, F3 = 1.5;
const double A2 = 0.9;

// MRT matrices with the reference's literal values (include/globalParameters.hpp:154-175)
const double M[81] = {1., 1., 1., 1., 1., 1., 1., 1., 1., -4., -1., -1., -1., -1., 2., 2., 2., 2., 4., -2., -2., -2., -2., 1., 1.,
                      1., 1., 0., 1., 0., -1., 0., 1., -1., -1., 1., 0., -2., 0., 2., 0., 1., -1., -1., 1., 0., 0., 1., 0., -1.,
                      1., 1., -1., -1., 0., 0., -2., 0., 2., 1., 1., -1., -1., 0., 1., -1., 1., -1., 0., 0., 0., 0., 0., 0.,
                      0., 0., 0., 1., -1., 1., -1.};
const double Minv[81] = {
    0.111111111111111, -0.111111111111111, 0.111111111111111, 0.0, -0.0, -0.0, -0.0, 0.0, 0.0,
    0.111111111111111, -0.027777777777778, -0.055555555555556, 0.166666666666667, -0.166666666666667, 0.0, 0.0, 0.25, -0.0,
    0.111111111111111, -0.027777777777778, -0.055555555555556, -0.0, -0.0, 0.166666666666667, -0.166666666666667, -0.25, 0.0,
    0.111111111111111, -0.027777777777778, -0.055555555555556, -0.166666666666667, 0.166666666666667, -0.0, -0.0, 0.25, -0.0,
    0.111111111111111, -0.027777777777778, -0.055555555555556, 0.0, 0.0, -0.166666666666667, 0.166666666666667, -0.25, -0.0,
    0.111111111111111, 0.055555555555556, 0.027777777777778, 0.166666666666667, 0.083333333333333, 0.166666666666667, 0.083333333333333, 0.0, 0.25,
    0.111111111111111, 0.055555555555556, 0.027777777777778, -0.166666666666667, -0.083333333333333, 0.166666666666667, 0.083333333333333, 0.0, -0.25,
    0.111111111111111, 0.055555555555556, 0.027777777777778, -0.166666666666667, -0.083333333333333, -0.166666666666667, -0.083333333333333, 0.0, 0.25,
    0.111111111111111, 0.055555555555556, 0.027777777777778, 0.166666666666667, 0.083333333333333, -0.166666666666667, -0.083333333333333, 0.0, -0.25};

// include/coreLB.hpp:634-643
void matmul(const double *a, const double *b, double *c)
{
    for (int u = 0; u < NC; u++)
    {
        c[u] = 0;
        for (int v = 0; v < NC; v++) c[u] += a[NC * u + v] * b[v];
    }
}

struct Oracle
{
    OracleParams p;
    int n, maxLevel;
    int64_t N;
    std::vector<int32_t> x, y, level, type, is_buffer, bnd;
    std::vector<int64_t> conn;
    std::vector<double> taus, kn;
    std::vector<int64_t> streamID, streamLOC, boundaryID, periodicID, periodicI2;
    std::vector<int32_t> streamIC, boundaryIC, periodicIC;
    std::map<int, std::vector<std::vector<int64_t>>> coarseBuffer, fineBuffer;
    int64_t inlet, inlet2, outlet, outlet2;
    std::vector<std::vector<int>> sfIC, bfIC;
    std::vector<std::vector<int64_t>> sfI2;
    // state
    std::vector<double> rho, rho_old, ux, uy, usq, usq_old, f, fb, ftemp, feq, fneq, psi, Fx, Fy;
    std::vector<std::vector<int>> icsr;
    std::vector<std::vector<double>> xy_norm;
    double diff = 1.0;
    std::vector<double> diffs;
    int t = 0;

    double tau_q(double ts) const { return 0.5 + (3.0 + M_PI * (2.0 * ts - 1.0) * (2.0 * ts - 1.0) * A2) / (8.0 * (2.0 * ts - 1.0)); }
    double tau_d_mrt(int64_t k) const
    {
        return 0.5 + (3.0 / 2.0) * std::sqrt(3.0) * 1.0 /
                         std::pow((1.0 / std::sqrt(p.mfp / p.Cl * 1.0 / (1.0 + 2.0 * kn[k]))) * 2.0, 2.0);
    }

    // include/coreLB.hpp:381-417
    void initialize(const double *rho_init)
    {
        size_t nn = (size_t)N;
        rho.assign(nn, p.rhoin);
        if (rho_init) rho.assign(rho_init, rho_init + N);
        rho_old.assign(nn, 0);
        ux.assign(nn, 0);
        uy.assign(nn, 0);
        usq.assign(nn, 0);
        usq_old.assign(nn, 0);
        f.assign(nn * NC, 0);
        feq.assign(nn * NC, 0);
        fb.assign(nn * NC, 0);
        ftemp.assign(nn * NC, 0);
        fneq.assign(nn * NC, 0);
        psi.assign(nn, 0);
        Fx.assign(nn, 0);
        Fy.assign(nn, 0);
        for (int64_t k = 0; k < N; k++)
            for (int ic = 0; ic < NC; ic++)
                f[k * NC + ic] = W[ic] * rho[k] *
                                 (1.0 + F1 * (EX[ic] * ux[k] + EY[ic] * uy[k]) +
                                  F2 * std::pow(EX[ic] * ux[k] + EY[ic] * uy[k], 2) - F3 * usq[k]);
        macroscopic();
    }

    // include/coreLB.hpp:420-430
    void equilibrium()
    {
#pragma omp parallel for
        for (int64_t k = 0; k < N; k++)
            for (int ic = 0; ic < NC; ic++)
                feq[k * NC + ic] = W[ic] * rho[k] *
                                   (1.0 + F1 * (EX[ic] * ux[k] + EY[ic] * uy[k]) +
                                    F2 * std::pow(EX[ic] * ux[k] + EY[ic] * uy[k], 2) - F3 * usq[k]);
    }

    // include/coreLB.hpp:646-675
    void regularize()
    {
#pragma omp parallel for
        for (int64_t k = 0; k < N; k++)
        {
            double pc[4] = {0, 0, 0, 0};
            int64_t k_ic = k * NC;
            for (int ic = 0; ic < NC; ic++)
            {
                double ccr[4] = {(double)(EX[ic] * EX[ic]), (double)(EX[ic] * EY[ic]), (double)(EX[ic] * EY[ic]),
                                 (double)(EY[ic] * EY[ic])};
                for (int u = 0; u < 4; u++) pc[u] += (f[k_ic + ic] - feq[k_ic + ic]) * ccr[u];
            }
            for (int ic = 0; ic < NC; ic++)
            {
                double H2[4] = {EX[ic] * EX[ic] / CS2 - 1, EX[ic] * EY[ic] / CS2, EX[ic] * EY[ic] / CS2,
                                EY[ic] * EY[ic] / CS2 - 1};
                fneq[k_ic + ic] = W[ic] * (1. / (2. * CS2)) * (pc[0] * H2[0] + pc[1] * H2[1] + pc[2] * H2[2] + pc[3] * H2[3]);
            }
        }
    }

    void relax(int64_t k, double td, const double *in, double *out) const
    {
        double R[9] = {1.0 / 1.0, 1.0 / 1.1, 1.0 / 1.2, 1.0 / td, 1.0 / tau_q(taus[k]),
                       1.0 / td,  1.0 / tau_q(taus[k]), 1.0 / taus[k], 1.0 / taus[k]};
        double m[9], mr[9];
        matmul(M, in, m);
        for (int u = 0; u < NC; u++) mr[u] = R[u] * m[u];
        matmul(Minv, mr, out);
    }

    // include/coreLB.hpp:744-792
    void collide_rmrt(int lvl)
    {
        regularize();
#pragma omp parallel for
        for (int64_t k = 0; k < N; k++)
        {
            if (level[k] != lvl) continue;
            double d[9];
            relax(k, 1.0, &fneq[k * NC], d);
            for (int ic = 0; ic < NC; ic++) f[k * NC + ic] = feq[k * NC + ic] + fneq[k * NC + ic] - d[ic];
        }
    }
    // include/coreLB.hpp:694-742
    void collide_mrt(int lvl)
    {
#pragma omp parallel for
        for (int64_t k = 0; k < N; k++)
        {
            if (level[k] != lvl) continue;
            double a[9], d[9];
            for (int ic = 0; ic < NC; ic++) a[ic] = f[k * NC + ic] - feq[k * NC + ic];
            relax(k, tau_d_mrt(k), a, d);
            for (int ic = 0; ic < NC; ic++) f[k * NC + ic] = f[k * NC + ic] - d[ic];
        }
    }
    // include/coreLB.hpp:678-691
    void collide_bgk(int lvl)
    {
        const double tau_srt = 1.0;
        for (int64_t k = 0; k < N; k++)
            if (level[k] == lvl)
                for (int ic = 0; ic < NC; ic++)
                    f[k * NC + ic] = f[k * NC + ic] - 1.0 / tau_srt * (f[k * NC + ic] - feq[k * NC + ic]);
    }
    void collide(int lvl)
    {
        if (p.collision == 2) collide_rmrt(lvl);
        else if (p.collision == 1) collide_mrt(lvl);
        else collide_bgk(lvl);
    }

    // include/coreLB.hpp:1233-1246, 834-856
    void zero_down(int lvl)
    {
#pragma omp parallel for
        for (int64_t i = 0; i < N; i++)
            if (level[i] == lvl)
                for (int ic = 0; ic < NC; ic++) f[i * NC + ic] = 0;
    }
    void stream(int lvl)
    {
#pragma omp parallel for
        for (int64_t i = 0; i < (int64_t)streamID.size(); i++)
            if (level[streamID[i]] == lvl) f[streamLOC[i] * NC + streamIC[i]] = ftemp[streamID[i] * NC + streamIC[i]];
    }
    int icsr_of(int64_t c, int q) const { return bnd[c] >= 0 ? icsr[bnd[c]][q] : OPPO[q]; }
    // include/coreLB.hpp:918-933 (serial: the += on one cell's populations is order-sensitive)
    void srbb(int lvl)
    {
        for (size_t i = 0; i < boundaryID.size(); i++)
        {
            int64_t c = boundaryID[i];
            if (level[c] != lvl) continue;
            double r = bnd[c] < 0 ? 1.0 : 0.4987 * std::pow(kn[c], -0.131) - 0.25;
            int q = boundaryIC[i];
            f[c * NC + OPPO[q]] += r * ftemp[c * NC + q];
            f[c * NC + icsr_of(c, q)] += (1 - r) * ftemp[c * NC + q];
        }
    }
    // include/coreLB.hpp:936-967
    void mdbb(int lvl)
    {
        for (size_t i = 0; i < boundaryID.size(); i++)
        {
            int64_t k1 = boundaryID[i];
            if (level[k1] != lvl) continue;
            int k2 = boundaryIC[i];
            double nx = bnd[k1] >= 0 ? xy_norm[bnd[k1]][0] : 0.0, ny = bnd[k1] >= 0 ? xy_norm[bnd[k1]][1] : 0.0;
            double kno = 0, kdeno = 0;
            for (int ic = 0; ic < NC; ic++)
            {
                double cn = EY[ic] * ny + EX[ic] * nx;
                if (cn > 0) kdeno += feq[k1 * NC + ic];
                else if (cn < 0) kno += fb[k1 * NC + ic];
            }
            double r = bnd[k1] < 0 ? 1.0 : 0.3222 * std::pow(kn[k1], -0.217) - 0.25;
            f[k1 * NC + OPPO[k2]] = r * ftemp[k1 * NC + k2] + (1 - r) * kno / kdeno * feq[k1 * NC + OPPO[k2]];
        }
    }
    // include/coreLB.hpp:859-865
    void bb(int lvl)
    {
        for (size_t i = 0; i < boundaryID.size(); i++)
            if (level[boundaryID[i]] == lvl)
                f[boundaryID[i] * NC + OPPO[boundaryIC[i]]] = ftemp[boundaryID[i] * NC + boundaryIC[i]];
    }
    // include/coreLB.hpp:969-977
    void periodic(int lvl)
    {
        for (size_t i = 0; i < periodicID.size(); i++)
            if (level[periodicID[i]] == lvl) f[periodicI2[i] * NC + periodicIC[i]] = ftemp[periodicID[i] * NC + periodicIC[i]];
    }
    void walls(int lvl)
    {
        if (p.wall == 2) srbb(lvl);
        else if (p.wall == 1) mdbb(lvl);
        else bb(lvl);
    }

    // include/coreLB.hpp:1018-1054
    void macroscopic()
    {
#pragma omp parallel for
        for (int64_t i = 0; i < N; i++)
        {
            double jx = 0, jy = 0;
            rho[i] = 0;
            for (int ic = 0; ic < NC; ic++)
            {
                rho[i] += f[i * NC + ic];
                jx += f[i * NC + ic] * EX[ic];
                jy += f[i * NC + ic] * EY[ic];
            }
            ux[i] = jx / rho[i] + p.fbody / (2.0 * rho[i]) * std::pow(2.0, level[i] - 1);
            uy[i] = jy / rho[i];
            usq[i] = ux[i] * ux[i] + uy[i] * uy[i];
        }
    }
    // include/coreLB.hpp:1056-1067
    void density()
    {
        for (int64_t i = 0; i < N; i++)
        {
            rho[i] = 0;
            for (int ic = 0; ic < NC; ic++) rho[i] += f[i * NC + ic];
        }
    }
    // include/coreLB.hpp:1069-1099
    void velocity()
    {
        for (int64_t i = 0; i < N; i++)
        {
            double jx = 0, jy = 0;
            for (int ic = 0; ic < NC; ic++)
            {
                jx += f[i * NC + ic] * EX[ic];
                jy += f[i * NC + ic] * EY[ic];
            }
            ux[i] = jx / rho[i] + Fx[i] / (2.0 * rho[i]) * std::pow(2.0, level[i] - 1);
            uy[i] = jy / rho[i] + Fy[i] / (2.0 * rho[i]) * std::pow(2.0, level[i] - 1);
            usq[i] = ux[i] * ux[i] + uy[i] * uy[i];
        }
    }
    // include/coreLB.hpp:515-531 (psi_form 0); psi_form 1: rho_psi (1 - exp(-rho / rho_psi))
    void pseudo_potential()
    {
        const double b_lu = 2.0 / 21.0, R_lu = 1.0, Mw_lu = 1.0;
        for (int64_t i = 0; i < N; i++)
        {
            if (p.psi_form == 1)
            {
                psi[i] = p.rho_psi * (1.0 - std::exp(-rho[i] / p.rho_psi));
                continue;
            }
            double md = rho[i] / Mw_lu;
            double acc = (md * R_lu * p.T_lu / (1 - b_lu * md) -
                          p.a_alpha_lu * md * md / (1 + 2 * b_lu * md - b_lu * b_lu * md * md) - (1.0 / 3.0) * rho[i]) /
                         (3.0 * p.g_ff);
            psi[i] = acc < 0 ? acc : std::sqrt(acc);
        }
    }
    // include/coreLB.hpp:533-566
    void forces()
    {
        for (int64_t i = 0; i < N; i++)
        {
            double fxf = 0, fyf = 0, fxw = 0, fyw = 0;
            for (size_t k = 0; k < sfIC[i].size(); k++)
            {
                int c = sfIC[i][k];
                int64_t nx = sfI2[i][k];
                fxf += (-6.0) * p.g_ff * psi[i] * WF[c] * psi[nx] * EX[c];
                fyf += (-6.0) * p.g_ff * psi[i] * WF[c] * psi[nx] * EY[c];
            }
            for (size_t k = 0; k < bfIC[i].size(); k++)
            {
                int c = bfIC[i][k];
                fxw += (-1.0) * p.g_fs * psi[i] * psi[i] * WF[c] * EX[c];
                fyw += (-1.0) * p.g_fs * psi[i] * psi[i] * WF[c] * EY[c];
            }
            Fx[i] = fxf + fxw + p.fbody;
            Fy[i] = fyf + fyw;
        }
    }
    // include/coreLB.hpp:568-630
    void source()
    {
        for (int64_t k = 0; k < N; k++)
        {
            double uF[4] = {ux[k] * Fx[k], ux[k] * Fy[k], uy[k] * Fx[k], uy[k] * Fy[k]};
            double S[9];
            for (int ic = 0; ic < NC; ic++)
            {
                double cDotF = EX[ic] * Fx[k] + EY[ic] * Fy[k];
                double ccs[4] = {(double)EX[ic] * EX[ic] - CS2, (double)EX[ic] * EY[ic], (double)EY[ic] * EX[ic],
                                 (double)EY[ic] * EY[ic] - CS2};
                S[ic] = W[ic] * (cDotF / CS2 + (uF[0] * ccs[0] + uF[2] * ccs[1] + uF[1] * ccs[2] + uF[3] * ccs[3]) / (CS2 * CS2));
            }
            double td = tau_d_mrt(k), tq = tau_q(taus[k]);
            double R[9] = {1.0, 1.0 / 1.1, 1.0 / 1.2, 1.0 / td, 1.0 / tq, 1.0 / td, 1.0 / tq, 1.0 / taus[k], 1.0 / taus[k]};
            double m[9], mr[9], d[9];
            matmul(M, S, m);
            for (int u = 0; u < NC; u++) mr[u] = (1.0 - 0.5 * R[u]) * m[u];
            matmul(Minv, mr, d);
            for (int ic = 0; ic < NC; ic++) f[k * NC + ic] = f[k * NC + ic] + d[ic];
        }
    }
    // include/coreLB.hpp:980-1009
    void inlet_outlet()
    {
        if (inlet >= 0)
        {
            f[inlet * NC + 1] = W[1] * p.rhoin;
            f[inlet * NC + 5] = W[2] * p.rhoin;
            f[inlet * NC + 8] = W[2] * p.rhoin;
        }
        if (outlet >= 0)
        {
            f[outlet * NC + 3] = W[1] * p.rhoin;
            f[outlet * NC + 6] = W[2] * p.rhoin;
            f[outlet * NC + 7] = W[2] * p.rhoin;
        }
    }
    // include/coreLB.hpp:1248-1267
    void velocity_difference()
    {
        double s1 = 0, s2 = 0;
        for (int64_t i = 0; i < N; i++)
        {
            s1 += std::abs(std::sqrt(usq[i]) - std::sqrt(usq_old[i]));
            s2 += std::sqrt(usq[i]);
        }
        diff = s1 / s2;
        diffs.push_back(diff);
    }
    // include/coreLB.hpp:1269-1283
    void density_difference()
    {
        double m = 0.0;
        for (int64_t i = 0; i < N; i++)
        {
            double d = std::abs(rho[i] - rho_old[i]) / rho_old[i];
            if (d > m) m = d;
        }
        if (m < 1.0e-15) m = 1.0e-5;
        diff = m;
        diffs.push_back(diff);
    }

    // include/coreLB.hpp:1101-1231, with defined meanings where the reference
    // reads outside its arrays: a missing coarse child is left out of the mean;
    // a wall/missing neighbour of a fine-buffer parent takes its periodic
    // lattice position and the parent's own populations.  A wall link of a cell
    // without boundary type (reference: ifStream[-1]) is a full bounce-back.
    void interpolate(int l1, int l2)
    {
        int key = l2 * 10 + l1;
        for (auto &cells : coarseBuffer[key])
        {
            double tf = 0;
            int cnt = 0;
            for (int ch = 1; ch < 5; ch++)
                if (cells[ch] >= 0)
                {
                    tf += taus[cells[ch]];
                    cnt++;
                }
            if (cnt == 0) continue;
            tf = tf / cnt;
            double tc = taus[cells[0]];
            for (int ic = 0; ic < NC; ic++)
            {
                double avg = 0;
                for (int ch = 1; ch < 5; ch++)
                    if (cells[ch] >= 0) avg += f[cells[ch] * NC + ic];
                avg = avg / cnt;
                f[cells[0] * NC + ic] = feq[cells[0] * NC + ic] + 2 * tc / tf * (avg - feq[cells[0] * NC + ic]);
            }
        }
        double parent_shift = std::pow(2.0, l2 - 2) - 0.5;
        double child_shift = (l1 == 1) ? 0 : std::pow(2.0, l1 - 2) - 0.5;
        key = l1 * 10 + l2;
        const int top_order[9] = {7, 4, 8, 3, 0, 1, 6, 2, 5};
        const int bottom_order[9] = {6, 2, 5, 3, 0, 1, 7, 4, 8};
        for (auto &cells : fineBuffer[key])
        {
            int64_t pc = cells[0];
            int64_t pconn[9];
            double X[9], Y[9];
            double thr = std::pow(2, level[pc] - 1);
            for (int ic = 0; ic < NC; ic++)
            {
                int64_t nb = conn[pc * 9 + ic];
                pconn[ic] = nb >= 0 ? nb : pc;
                // a wall / missing neighbour sits at its periodic lattice position
                int yn = nb >= 0 ? y[nb] : (int)(((y[pc] + EY[ic] * (int)thr) % n + n) % n);
                int xn = nb >= 0 ? x[nb] : (int)(((x[pc] + EX[ic] * (int)thr) % n + n) % n);
                if (std::abs(y[pc] - yn) > thr && y[pc] - yn < 0) X[ic] = y[pc] + parent_shift + 1 - 2;
                else if (std::abs(y[pc] - yn) > thr && y[pc] - yn > 0) X[ic] = y[pc] + parent_shift + 1 + 2;
                else X[ic] = yn + parent_shift + 1;
                if (std::abs(x[pc] - xn) > thr && x[pc] - xn < 0) Y[ic] = x[pc] + parent_shift + 1 - 2;
                else if (std::abs(x[pc] - xn) > thr && x[pc] - xn > 0) Y[ic] = x[pc] + parent_shift + 1 + 2;
                else Y[ic] = xn + parent_shift + 1;
            }
            std::vector<double> Xs(X, X + 9), Ys(Y, Y + 9);
            std::sort(Xs.begin(), Xs.end());
            Xs.erase(std::unique(Xs.begin(), Xs.end()), Xs.end());
            std::sort(Ys.begin(), Ys.end());
            Ys.erase(std::unique(Ys.begin(), Ys.end()), Ys.end());
            alglib::real_1d_array xa, ya, Z;
            xa.setlength(3);
            ya.setlength(3);
            Z.setlength(9);
            bool top = y[pc] < n / 2;
            for (size_t i = 0; i < Xs.size() && i < 3; i++) ya[i] = top ? Xs[i] : Xs[Xs.size() - i - 1];
            for (size_t i = 0; i < Ys.size() && i < 3; i++) xa[i] = Ys[i];
            double tc = taus[pc];
            for (int ic = 0; ic < NC; ic++)
            {
                for (int k = 0; k < NC; k++) Z[k] = f[pconn[top ? top_order[k] : bottom_order[k]] * NC + ic];
                alglib::spline2dinterpolant s;
                alglib::spline2dbuildbicubicv(xa, 3, ya, 2, Z, 1, s);
                for (int ch = 1; ch < 5; ch++)
                {
                    int64_t c = cells[ch];
                    double fi = alglib::spline2dcalc(s, x[c] + child_shift + 1, y[c] + child_shift + 1);
                    f[c * NC + ic] = feq[c * NC + ic] + taus[c] / (2 * tc) * (fi - feq[c * NC + ic]);
                }
            }
        }
    }

    // include/coreLB.hpp:1310-1331
    void evolution(int lvl)
    {
        int rep = (int)std::pow(2, maxLevel - lvl);
        for (int i = 0; i < rep; i++)
        {
            fb = f;
            collide(lvl);
            ftemp = f;
            zero_down(lvl);
            stream(lvl);
            walls(lvl);
            periodic(lvl);
        }
        if (lvl > 1) evolution(lvl - 1);
        if (lvl != maxLevel) interpolate(lvl, lvl + 1);
    }

    // include/mantiisApp.hpp:239-246
    void transport_step()
    {
        usq_old = usq;
        equilibrium();
        evolution(maxLevel);
        macroscopic();
        velocity_difference();
    }
    // include/mantiisApp.hpp:267-284 (the coupling phase of the coupled run)
    void coupled_step()
    {
        rho_old = rho;
        density();
        pseudo_potential();
        forces();
        velocity();
        equilibrium();
        collide_rmrt(1);
        source();
        ftemp = f;
        zero_down(1);
        stream(1);
        srbb(1);
        periodic(1);
        velocity_difference(); // usq_old is never updated in this run: the ratio is 1
    }
    // the coupled run (include/mantiisApp.hpp:376-392): up to 100 adsorption
    // steps without body force (ended early by the residual test), a reset of
    // u, rho and f_eq, then coupling steps
    int coupled_a = 0;
    bool coupled_b = false;
    void coupled_run_step()
    {
        if (coupled_b)
        {
            coupled_step();
            return;
        }
        const double fb = p.fbody;
        p.fbody = 0.0;
        adsorption_step();
        p.fbody = fb;
        coupled_a++;
        if (coupled_a >= 100 || diff < p.tol)
        {
            coupled_b = true;
            std::fill(ux.begin(), ux.end(), 0.0);
            std::fill(rho.begin(), rho.end(), p.rhoin);
            std::fill(feq.begin(), feq.end(), 0.0);
        }
    }
    // include/mantiisApp.hpp:248-265
    void adsorption_step()
    {
        rho_old = rho;
        density();
        pseudo_potential();
        forces();
        velocity();
        equilibrium();
        collide_mrt(1);
        source();
        ftemp = f;
        zero_down(1);
        stream(1);
        bb(1);
        periodic(1);
        inlet_outlet();
        density_difference();
    }
};
} // namespace

extern "C" {

void *oracle_create(const OracleGrid *g, const OracleParams *p, const double *rho_init)
{
    Oracle *o = new Oracle();
    o->p = *p;
    o->n = g->n;
    o->maxLevel = g->max_level;
    o->N = g->n_cells;
    size_t N = (size_t)g->n_cells;
    o->x.assign(g->x, g->x + N);
    o->y.assign(g->y, g->y + N);
    o->level.assign(g->level, g->level + N);
    o->type.assign(g->type, g->type + N);
    o->is_buffer.assign(g->is_buffer, g->is_buffer + N);
    o->bnd.assign(g->bnd, g->bnd + N);
    o->conn.assign(g->conn, g->conn + N * 9);
    o->taus.assign(g->tau, g->tau + N);
    o->kn.assign(g->kn, g->kn + N);
    o->streamID.assign(g->stream_id, g->stream_id + g->n_stream);
    o->streamIC.assign(g->stream_ic, g->stream_ic + g->n_stream);
    o->streamLOC.assign(g->stream_loc, g->stream_loc + g->n_stream);
    o->boundaryID.assign(g->wall_id, g->wall_id + g->n_wall);
    o->boundaryIC.assign(g->wall_ic, g->wall_ic + g->n_wall);
    o->periodicID.assign(g->per_id, g->per_id + g->n_per);
    o->periodicI2.assign(g->per_i2, g->per_i2 + g->n_per);
    o->periodicIC.assign(g->per_ic, g->per_ic + g->n_per);
    for (int64_t r = 0; r < g->n_coarse; r++)
        o->coarseBuffer[(int)g->coarse_rows[r * 6]].push_back(
            std::vector<int64_t>(g->coarse_rows + r * 6 + 1, g->coarse_rows + r * 6 + 6));
    for (int64_t r = 0; r < g->n_fine; r++)
        o->fineBuffer[(int)g->fine_rows[r * 6]].push_back(std::vector<int64_t>(g->fine_rows + r * 6 + 1, g->fine_rows + r * 6 + 6));
    o->inlet = (g->inlet >= 0 && g->outlet >= 0) ? g->inlet : -1;
    o->outlet = (g->inlet >= 0 && g->outlet >= 0) ? g->outlet : -1;
    o->inlet2 = g->inlet2;
    o->outlet2 = g->outlet2;
    // Shan-Chen force lists (include/coreLB.hpp:293-356): stream + periodic links, wall links
    o->sfIC.assign(N, {});
    o->sfI2.assign(N, {});
    o->bfIC.assign(N, {});
    // per cell in direction order, as the constructor builds them
    std::vector<std::vector<std::pair<int, int64_t>>> s(N), b(N);
    for (int64_t i = 0; i < g->n_stream; i++) s[g->stream_id[i]].push_back({g->stream_ic[i], g->stream_loc[i]});
    for (int64_t i = 0; i < g->n_per; i++) s[g->per_id[i]].push_back({g->per_ic[i], g->per_i2[i]});
    for (int64_t i = 0; i < g->n_wall; i++) b[g->wall_id[i]].push_back({g->wall_ic[i], -1});
    for (size_t i = 0; i < N; i++)
    {
        std::stable_sort(s[i].begin(), s[i].end(), [](auto &a, auto &c) { return a.first < c.first; });
        for (auto &e : s[i])
        {
            o->sfIC[i].push_back(e.first);
            o->sfI2[i].push_back(e.second);
        }
        for (auto &e : b[i]) o->bfIC[i].push_back(e.first);
    }
    o->icsr.assign(ORACLE_N_BND_TYPES, std::vector<int>(9));
    o->xy_norm.assign(ORACLE_N_BND_TYPES, std::vector<double>(2));
    for (int t = 0; t < ORACLE_N_BND_TYPES; t++)
    {
        for (int q = 0; q < 9; q++) o->icsr[t][q] = ORACLE_ICSR[t][q];
        o->xy_norm[t][0] = ORACLE_XY_NORM[t][0];
        o->xy_norm[t][1] = ORACLE_XY_NORM[t][1];
    }
    o->initialize(rho_init);
    return o;
}

int oracle_run(void *h, int n, int break_on_tol)
{
    Oracle *o = (Oracle *)h;
    int done = 0;
    for (int i = 0; i < n; i++)
    {
        if (o->p.simulation == 2)
        {
            // the first phase ends on the residual test, the coupling phase runs on
            const bool in_a = !o->coupled_b;
            o->coupled_run_step();
            done++;
            if (!in_a && break_on_tol && o->diff < o->p.tol) break;
            o->t++;
            continue;
        }
        if (o->p.simulation == 1) o->adsorption_step();
        else o->transport_step();
        done++;
        if (break_on_tol && o->diff < o->p.tol) break;
        o->t++;
    }
    return done;
}

void oracle_fields(void *h, double *rho, double *ux, double *uy, double *f)
{
    Oracle *o = (Oracle *)h;
    if (rho) std::copy(o->rho.begin(), o->rho.end(), rho);
    if (ux) std::copy(o->ux.begin(), o->ux.end(), ux);
    if (uy) std::copy(o->uy.begin(), o->uy.end(), uy);
    if (f) std::copy(o->f.begin(), o->f.end(), f);
}

int64_t oracle_residuals(void *h, double *out, int64_t cap)
{
    Oracle *o = (Oracle *)h;
    int64_t n = (int64_t)o->diffs.size();
    if (out)
        for (int64_t i = 0; i < std::min(n, cap); i++) out[i] = o->diffs[i];
    return n;
}

void oracle_destroy(void *h) { delete (Oracle *)h; }

int oracle_threads(int n)
{
#ifdef _OPENMP
    int prev = omp_get_max_threads();
    if (n > 0) omp_set_num_threads(n);
    return prev;
#else
    (void)n;
    return 1;
#endif
}
}
