#include "units.hpp"

#include <cmath>
#include <limits>
#include <vector>

namespace mantiis
{
namespace
{
// Largest real root of a x^3 + b x^2 + c x + d = 0 by Cardano's formula, the
// one-real-root branch only (include/utils.hpp:571-600; the other branches
// return no root there, and the maximum of an empty set is DBL_MIN,
// include/utils.hpp:226-239).
double cardano_max_root(double a, double b, double c, double d)
{
    std::vector<double> roots;
    double p = (3 * a * c - b * b) / (3 * a * a);
    double q = (2 * b * b * b - 9 * a * b * c + 27 * a * a * d) / (27 * a * a * a);
    double delta = -4 * p * p * p - 27 * q * q;
    if (delta < 0)
    {
        double u1 = -q / 2 + std::sqrt(q * q / 4 + p * p * p / 27);
        double u2 = -q / 2 - std::sqrt(q * q / 4 + p * p * p / 27);
        double t = std::pow(u1, 1.0 / 3.0) + std::pow(u2, 1.0 / 3.0);
        roots.push_back(t - b / (3 * a));
    }
    double m = std::numeric_limits<double>::min();
    for (double r : roots)
        if (r > m) m = r;
    return m;
}
} // namespace

void UnitSystem::recompute()
{
    const double NA = 6.02214076e23;
    const double R_EOS = 8.31446;
    const double Rs_lu = R_lu / Mw_lu;
    double k = 0.37464 + 1.54226 * omega - 0.26992 * std::pow(omega, 2);
    alpha = std::pow((1 + k * (1 - std::sqrt(T_phy / Tc_phy))), 2);
    a_alpha_lu = a_lu * alpha;
    double Rs = R_EOS / Mw;

    double a = 0.45724 * (R_EOS * Tc_phy) * (R_EOS * Tc_phy) / Pc_phy;
    double aG = a * alpha;
    double bG = 0.07780 * R_EOS * Tc_phy / Pc_phy;
    double AG = aG * P_phy / (R_EOS * R_EOS) / (T_phy * T_phy);
    double BG = bG * P_phy / R_EOS / T_phy;

    double ZG2 = BG - 1;
    double ZG1 = AG - 3 * (BG * BG) - 2 * BG;
    double ZG0 = BG * BG * BG + (BG * BG) - AG * BG;
    double ZG = cardano_max_root(1.0, ZG2, ZG1, ZG0);
    double vG = ZG * R_EOS * T_phy / P_phy;
    double rho_phy_mol = 1 / vG;
    rho_phy = rho_phy_mol * Mw;

    double C_Rs = Rs / Rs_lu;
    double b_Rs = 0.07780 * Rs * Tc_phy / Pc_phy;
    double a_Rs = 0.45724 * std::pow((Rs * Tc_phy), 2) / Pc_phy;
    double C_as = a_Rs / a_lu;
    double C_bs = b_Rs / b_lu;
    double C_aob = C_as / C_bs;
    Ct = Cl / std::sqrt(C_aob);
    CT = 1 / (C_Rs / std::pow(Cl, 2) * std::pow(Ct, 2));
    T_lu = T_phy / CT;
    double C_Mw = Mw / Mw_lu;
    Cm = std::pow(Cl, 3) / C_bs;
    Crho = Cm / (Cl * Cl * Cl);
    Cn = Cm / C_Mw;
    Cu = Cl / Ct;
    Cf = Cm / (std::pow(Ct, 2) * std::pow(Cl, 2));
    Crho_mol = Cn / std::pow(Cl, 3);
    rhoin = rho_phy / Crho;

    mfp = 1.0 / (std::sqrt(2.0) * Crho_mol * rhoin / Mw_lu * NA * M_PI * (2 * d_mol / 2.0 + 2 * d_mol / 2.0) *
                 (2 * d_mol / 2.0 + 2 * d_mol / 2.0));
}
} // namespace mantiis
