// Host-side set-up of the mock path: box/cosmology constants, the natural
// cubic spline of the input spectrum, the sigma(M) / barrier / mass-function
// tables of the halo finder and the sphere-shell offsets.  All of it is
// O(Nk^2 + Ncells) work done once per call on the host, in the reference's
// arithmetic (float where it stores floats, double where it computes in
// double).  Compiled with floating-point contraction off.
#pragma once
#include <stdint.h>
#include <stddef.h>
#include <vector>

namespace exh {

// exshalos_h.h:65-104 (cosmology, barrier, box), with the same float storage
struct BoxParams {
  float Om0, redshift, dc, rhoc, Hz, Omz, rhomz;
  float Lc, Mcell, L[3], Mtot, kl[3], Normx, Normk;
  int nd[3], nz2, nmin;
  size_t ng;
  int Nmin, seed, DO_EB;
  float a, beta, alpha;
  double Omz_d, Hz_d;
};

int setup_box(BoxParams* b, int ndx, int ndy, int ndz, float Lc, float Om0, float z, float dc, int Nmin,
              float a, float beta, float alpha, int seed);

// natural cubic spline, coefficients c (second derivative / 2)
struct Spline {
  std::vector<double> x, y, c;
  int init(const double* xs, const double* ys, int n);
  double eval(double q, int* status) const;
};

int ncells(const BoxParams& b);
// Compute_Sig + Compute_nh + Barrier table.  prec64 selects FP64 set-up.
int halo_tables(const BoxParams& b, const float* K, const float* P, int Nk, int prec64,
                std::vector<float>& Sig_grid, std::vector<float>& Btab, std::vector<double>& M,
                std::vector<double>& Int);
float barrier(const BoxParams& b, float S);
// smoothing ladder: n_radii log-spaced radii from Lc to R_max and the
// barrier B(sigma^2(R)) at each (sigma^2 by the FP64 trapezoid)
int ladder_tables(const BoxParams& b, const float* K, const float* P, int Nk, int n_radii, float R_max,
                  std::vector<float>& R, std::vector<float>& B);
// Gaussian-field amplitude sqrt(P(k)/2) per integer |n|^2 for a cubic box
int amplitude_table(const BoxParams& b, const float* K, const float* P, int Nk, std::vector<float>& A);
// cumulative cells per non-empty shell (find_halos.c:382-420), lmax = 10000
const std::vector<int>& cells_in_spheres();

}  // namespace exh
