// Physical-to-lattice unit system of the solver.
//
// Restates _GLOBAL_::recompute() (include/globalParameters.hpp:180-221) and the
// static initialisers above it (:50-132): the Peng-Robinson cubic for methane
// at (T, P), the conversion factors, the inlet density rho_in in lattice units
// and the mean free path.  The arithmetic is kept in the same order so rho_in
// and mfp are bit-identical to the reference's.
#pragma once

namespace mantiis
{
struct UnitSystem
{
    // inputs (Settings of include/mantiisApp.hpp:46-64 and _GLOBAL_ fluid data)
    double Cl = 1.0e-9;            // lattice spacing dx, m
    double T_phy = 300.0;          // K
    double P_phy = 2.0e6;          // Pa
    double Tc_phy = 190.564;       // methane critical temperature, K
    double Pc_phy = 4.5992 * 1.0e6;
    double d_mol = 3.800e-10;      // molecular diameter, m
    double omega = 0.011;          // acentric factor
    double Mw = 16.043 * 1.0e-3;   // kg/mol

    // derived
    double alpha = 0, a_alpha_lu = 0;
    double Ct = 0, CT = 0, T_lu = 0, Cm = 0, Crho = 0, Cn = 0, Cu = 0, Cf = 0, Crho_mol = 0;
    double rho_phy = 0;
    double rhoin = 0;  // inlet / initial density, lattice units
    double mfp = 0;    // mean free path, m

    // lattice PR-EOS constants and interaction strengths
    static constexpr double a_lu = 2.0 / 49.0;
    static constexpr double b_lu = 2.0 / 21.0;
    static constexpr double R_lu = 1.0;
    static constexpr double Mw_lu = 1.0;
    static constexpr double Gfs = -12.7;
    static constexpr double Gff = -1.0;
    static constexpr double A2 = 0.9;

    void recompute();
};
} // namespace mantiis
