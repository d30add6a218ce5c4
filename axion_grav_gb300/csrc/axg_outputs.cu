// axg_outputs.cu -- the reference program's text outputs, for C hosts.
//
// The reference writes its results from the host after each output time; a
// Fortran host of this library keeps those writers.  These give a C (or
// other non-Fortran) host the same files, formatted as the reference's
// edit descriptors format them:
//   <root>_string_wall_parameters.txt  (I,11E20.10e3)  evolve.f90:90,127,202
//   <root>_crho.txt                    (I,3E20.10e3)   evolve.f90:91,128
//   <root>_spectrum_<idx>.dat          (4E20.10e3)     spectrum.f90:278-285
//   <root>_covariance_<idx>.dat        (2I,E20.10e3)   spectrum.f90:294-302
//   <root>_gravspec_<idx>.dat          (5E20.10e3)     grav_waves.f90:308-316
//   <root>_eps.txt                     (2I,7E20.10e3)  spectrum.f90:1034-1035
// Integers take the Intel compiler's default I width for 4-byte integers
// (12); Ew.dEe writes 0.<d digits>E<sign><e digits>, the d significant
// digits correctly rounded from the double (round half to even on the exact
// decimal value, as printf's %e rounds it).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "axg_internal.h"

namespace {

constexpr int kIntWidth = 12;
constexpr double kMstarInHz = 2.435e18 * 1.5192488833521e24;  // potential.f90:13-23
constexpr double kRefTwoPi = 2 * 3.14159265359;                  // potential.f90:8

// E20.10e3 of x, 20 characters and a terminating zero in out[21]
void fortran_e(double x, char out[21]) {
  char body[32];
  if (std::isnan(x)) {
    std::snprintf(out, 21, "%20s", "NaN");
    return;
  }
  if (std::isinf(x)) {
    std::snprintf(out, 21, "%20s", x < 0 ? "-Infinity" : "Infinity");
    return;
  }
  const bool neg = std::signbit(x);
  if (x == 0) {
    std::snprintf(body, sizeof body, "%s0.0000000000E+000", neg ? "-" : "");
  } else {
    // d.ddddddddde+XX: ten significant digits, correctly rounded
    char e10[32];
    std::snprintf(e10, sizeof e10, "%.9e", std::fabs(x));
    const int exp10 = std::atoi(std::strchr(e10, 'e') + 1) + 1;  // 0.d... x 10^exp10
    char digits[11];
    digits[0] = e10[0];
    std::memcpy(digits + 1, e10 + 2, 9);
    digits[10] = 0;
    std::snprintf(body, sizeof body, "%s0.%sE%c%03d", neg ? "-" : "", digits, exp10 >= 0 ? '+' : '-',
                  exp10 >= 0 ? exp10 : -exp10);
  }
  std::snprintf(out, 21, "%20s", body);
}

std::string line(const int *ints, int ni, const double *reals, int nr) {
  std::string s;
  char buf[32];
  for (int i = 0; i < ni; ++i) {
    std::snprintf(buf, sizeof buf, "%*d", kIntWidth, ints[i]);
    s += buf;
  }
  for (int i = 0; i < nr; ++i) {
    fortran_e(reals[i], buf);
    s += buf;
  }
  s += '\n';
  return s;
}

int write_all(const std::string &path, const char *mode, const std::string &text) {
  FILE *f = std::fopen(path.c_str(), mode);
  if (!f) return axg_set_error(nullptr, AXG_ERR_IO, "cannot open " + path);
  const size_t w = std::fwrite(text.data(), 1, text.size(), f);
  const int c = std::fclose(f);
  if (w != text.size() || c != 0) return axg_set_error(nullptr, AXG_ERR_IO, "cannot write " + path);
  return AXG_OK;
}

std::string indexed(const char *root, const char *kind, int idx) {
  return std::string(root) + "_" + kind + "_" + std::to_string(idx) + ".dat";
}

}  // namespace

extern "C" int axg_write_spectrum(const char *root, int32_t idx, const double *wave, const double *power,
                                  const double *conv_per_mode, const double *count, int32_t nb) {
  if (!root || !wave || !power || !conv_per_mode || !count || nb < 0)
    return axg_set_error(nullptr, AXG_ERR_ARG, "axg_write_spectrum: null argument");
  std::string text;
  for (int i = 0; i < nb; ++i) {
    const double r[4] = {wave[i], power[i], conv_per_mode[i], count[i]};
    text += line(nullptr, 0, r, 4);
  }
  return write_all(indexed(root, "spectrum", idx), "w", text);
}

extern "C" int axg_write_covariance(const char *root, int32_t idx, const double *cov, int32_t nb) {
  if (!root || !cov || nb < 0) return axg_set_error(nullptr, AXG_ERR_ARG, "axg_write_covariance: null argument");
  std::string text;
  for (int i = 1; i <= nb; ++i)
    for (int j = 1; j <= i; ++j) {
      const int ij[2] = {i, j};
      text += line(ij, 2, &cov[(int64_t)i * (i - 1) / 2 + j - 1], 1);  // packed upper storage
    }
  return write_all(indexed(root, "covariance", idx), "w", text);
}

extern "C" int axg_write_gravspec(const char *root, int32_t idx, double tau, const double *wave, const double *power,
                                  const double *denom, int32_t nb, double tau_cr, double a_now) {
  if (!root || !wave || !power || !denom || nb < 0)
    return axg_set_error(nullptr, AXG_ERR_ARG, "axg_write_gravspec: null argument");
  const double fq = kMstarInHz / tau_cr / a_now / kRefTwoPi;  // grav_waves.f90:266
  std::string text;
  for (int i = 0; i < nb; ++i) {
    const double r[5] = {tau, wave[i], wave[i] * fq, power[i], denom[i]};
    text += line(nullptr, 0, r, 5);
  }
  return write_all(indexed(root, "gravspec", idx), "w", text);
}

extern "C" int axg_append_string_wall_line(const char *path, int32_t idx, double tau, double zeta_tau2,
                                           const double xi[3], const double area[3], const double vel[3]) {
  if (!path || !xi || !area || !vel) return axg_set_error(nullptr, AXG_ERR_ARG, "axg_append_string_wall_line");
  const double r[11] = {tau, zeta_tau2, xi[0], xi[1], xi[2], area[0], area[1], area[2], vel[0], vel[1], vel[2]};
  return write_all(path, "a", line(&idx, 1, r, 11));
}

extern "C" int axg_append_crho_line(const char *path, int32_t idx, double crho0, double crho1, double crho2) {
  if (!path) return axg_set_error(nullptr, AXG_ERR_ARG, "axg_append_crho_line");
  const double r[3] = {crho0, crho1, crho2};
  return write_all(path, "a", line(&idx, 1, r, 3));
}

extern "C" int axg_append_eps_line(const char *path, int32_t idx, int32_t idx2, double tau1, double tau2, double eps,
                                   double deps, const double crho1[2], const double crho2[2]) {
  if (!path || !crho1 || !crho2) return axg_set_error(nullptr, AXG_ERR_ARG, "axg_append_eps_line");
  const int ii[2] = {idx, idx2};
  const double r[7] = {tau1, tau2, (tau2 + tau1) / 2, eps, deps, crho2[0] - crho1[0],
                       std::sqrt(crho2[1] * crho2[1] + crho1[1] * crho1[1])};
  return write_all(path, "a", line(ii, 2, r, 7));
}
