// Stiffened-gas two-material mixture in the interface of the external
// core::eos::MieGruneisenMixture (the EOS itself is not in the reference tree;
// this is the same restatement as the oracle's, term for term).
#pragma once
#include <cmath>
#include <kalypsso/utils/config/ConfigMap.h>
namespace kalypsso { namespace core { namespace eos {
template <typename device_t>
class MieGruneisenMixture
{
public:
  double gamma[2], pinf[2], xi[2], gpx[2];
  MieGruneisenMixture(ConfigMap const & c)
  {
    for (int k = 0; k < 2; ++k)
    {
      const std::string sec = "material" + std::to_string(k) + "_mie_gruneisen_sg";
      gamma[k] = c.getReal(sec, "gamma", 1.4);
      pinf[k] = c.getReal(sec, "pinf", 0.0);
      xi[k] = 1.0 / (gamma[k] - 1.0);
      gpx[k] = gamma[k] * pinf[k] * xi[k];
    }
  }
  double S(double a0, double a1) const { return a0 * xi[0] + a1 * xi[1]; }
  double PI(double a0, double a1) const { return a0 * gpx[0] + a1 * gpx[1]; }
  double mixture_pressure(double rho, double eint, double a0, double a1, double, double) const
  {
    return (rho * eint - PI(a0, a1)) / S(a0, a1);
  }
  double mixture_specific_eint(double rho, double p, double a0, double a1, double, double) const
  {
    return (p * S(a0, a1) + PI(a0, a1)) / rho;
  }
  double mixture_sound_speed(double rho, double p, double a0, double a1, double, double) const
  {
    const double s = S(a0, a1);
    const double c2 = (p * (s + 1.0) + PI(a0, a1)) / (rho * s);
    return std::sqrt(std::fmax(c2, 0.0));
  }
  // bulk moduli of the Miller-Puckett source term: K_k = gamma_k (p + pinf_k),
  // 1 / Kbar = a0 / K0 + a1 / K1
  double material_bulk_modulus(int k, double p, double, double) const { return gamma[k] * (p + pinf[k]); }
  double mixture_bulk_modulus(double, double p, double a0, double a1, double ar0, double ar1) const
  {
    return 1.0 / (a0 / material_bulk_modulus(0, p, a0, ar0) + a1 / material_bulk_modulus(1, p, a1, ar1));
  }
};
} } }
