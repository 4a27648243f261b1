// Host-side set-up tables (see setup.h).  Reference formulas:
//   cosmology      src/exshalos/exshalos_h.c:43-57
//   box            src/exshalos/exshalos_h.c:69-106
//   sigma(R), S(M) src/exshalos/find_halos.c:4-44
//   f(sigma), I(M) src/exshalos/find_halos.c:47-93
//   barrier        src/exshalos/find_halos.c:200-212
//   sphere counts  src/exshalos/find_halos.c:382-420
// Expressions keep the reference's float/double mix term by term so that the
// tables are bit-identical to what the reference computes with the same libm.
#include "setup.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "../../include/exh_gb300.h"

namespace exh {

static const double kMmax = 1e+16;  // exshalos_h.h:47

// f(i) for i in [0, n) on up to hardware_concurrency threads; every index is
// computed by exactly one thread, so the results do not depend on the split.
template <class F>
static void parallel_for(int n, F f) {
  int nt = (int)std::min<unsigned>(std::max(1u, std::thread::hardware_concurrency()), 32u);
  nt = std::min(nt, std::max(1, n / 16));
  if (nt <= 1) {
    for (int i = 0; i < n; i++) f(i);
    return;
  }
  std::vector<std::thread> th;
  for (int t = 0; t < nt; t++)
    th.emplace_back([=]() {
      for (int i = t; i < n; i += nt) f(i);
    });
  for (auto& x : th) x.join();
}

// The reference calls the C <math.h> functions, which take and return double
// even for float arguments; these wrappers keep that promotion (the C++
// overloads would otherwise pick the float versions).
static inline double c_sqrt(double x) { return std::sqrt(x); }
static inline double c_pow(double x, double y) { return std::pow(x, y); }
static inline double c_sin(double x) { return std::sin(x); }
static inline double c_cos(double x) { return std::cos(x); }
static inline double c_exp(double x) { return std::exp(x); }
static inline double c_log10(double x) { return std::log10(x); }
static inline double c_log(double x) { return std::log(x); }

int setup_box(BoxParams* b, int ndx, int ndy, int ndz, float Lc, float Om0, float z, float dc, int Nmin,
              float a, float beta, float alpha, int seed) {
  std::memset(b, 0, sizeof(*b));
  b->Om0 = Om0;
  b->redshift = z;
  b->rhoc = 2.775e+11f;
  const double zp3 = c_pow(1.0 + (double)b->redshift, 3.0);
  b->Hz = (float)(100.0 * c_sqrt(b->Om0 * zp3 + (1.0 - b->Om0)));
  b->Omz = (float)(b->Om0 * zp3 / (b->Om0 * zp3 + (1.0 - b->Om0)));
  b->rhomz = b->Om0 * b->rhoc;
  b->dc = dc <= 0.0f ? (float)(1.686 * c_pow((double)b->Omz, 0.0055)) : dc;
  b->Omz_d = (double)Om0 * zp3 / ((double)Om0 * zp3 + (1.0 - (double)Om0));
  b->Hz_d = 100.0 * c_sqrt((double)Om0 * zp3 + (1.0 - (double)Om0));
  if (!(Lc > 0.0f && Lc < 100.0f)) return EXH_E_INVALID;    // Lc_MAX, exshalos_h.h:45
  b->nd[0] = ndx; b->nd[1] = ndy; b->nd[2] = ndz;
  b->ng = (size_t)ndx * (size_t)ndy * (size_t)ndz;
  b->nz2 = ndz / 2 + 1;
  b->Lc = Lc;
  b->Mcell = (float)(b->rhomz * c_pow((double)Lc, 3.0));
  for (int i = 0; i < 3; i++) b->L[i] = b->Lc * b->nd[i];
  b->Mtot = b->rhomz * b->L[0] * b->L[1] * b->L[2];
  for (int i = 0; i < 3; i++) b->kl[i] = (float)(2.0 * M_PI / b->L[i]);
  const float vol = b->L[0] * b->L[1] * b->L[2];
  b->Normx = (float)(1.0 / c_sqrt((double)vol));
  b->Normk = (float)(c_sqrt((double)vol) / (double)(ndx * ndy * ndz));
  b->nmin = std::min(ndx, std::min(ndy, ndz));
  b->Nmin = Nmin; b->seed = seed;
  b->a = a; b->beta = beta; b->alpha = alpha;
  b->DO_EB = (a == 1.0f && beta == 0.0f && alpha == 0.0f) ? 0 : 1;   // exshalos.c:737-740
  return EXH_OK;
}

int Spline::init(const double* xs, const double* ys, int n) {
  if (n < 3) return EXH_E_INVALID;
  for (int i = 0; i + 1 < n; i++)
    if (!(xs[i + 1] > xs[i])) return EXH_E_INVALID;
  x.assign(xs, xs + n);
  y.assign(ys, ys + n);
  c.assign(n, 0.0);
  const int m = n - 2;
  std::vector<double> d(m), r(m), o(m);
  for (int i = 0; i < m; i++) {
    const double h0 = xs[i + 1] - xs[i], h1 = xs[i + 2] - xs[i + 1];
    d[i] = 2.0 * (h0 + h1);
    o[i] = h1;
    r[i] = 3.0 * ((ys[i + 2] - ys[i + 1]) / h1 - (ys[i + 1] - ys[i]) / h0);
  }
  for (int i = 1; i < m; i++) {
    const double w = o[i - 1] / d[i - 1];
    d[i] = d[i] - w * o[i - 1];
    r[i] = r[i] - w * r[i - 1];
  }
  if (m > 0) c[m] = r[m - 1] / d[m - 1];
  for (int i = m - 2; i >= 0; i--) c[i + 1] = (r[i] - o[i] * c[i + 2]) / d[i];
  return EXH_OK;
}

double Spline::eval(double q, int* status) const {
  const int n = (int)x.size();
  if (q < x[0] || q > x[n - 1]) {
    if (status) *status = 1;
    return NAN;
  }
  size_t lo = 0, hi = (size_t)n - 1;
  while (hi > lo + 1) {
    const size_t mid = (hi + lo) / 2;
    if (x[mid] > q) hi = mid; else lo = mid;
  }
  const double xl = x[lo], dx = x[lo + 1] - xl, dy = y[lo + 1] - y[lo];
  const double c0 = c[lo], c1 = c[lo + 1];
  const double bb = dy / dx - dx * (c1 + 2.0 * c0) / 3.0;
  const double dd = (c1 - c0) / (3.0 * dx);
  const double t = q - xl;
  return y[lo] + t * (bb + t * (c0 + t * dd));
}

int ncells(const BoxParams& b) { return (int)std::floor(kMmax / b.Mcell); }

static float tophat_f(float k, float R) {
  return (float)(3.0 / (c_pow(k * R, 2)) * (c_sin(k * R) / (k * R) - c_cos(k * R)));
}
static double tophat_d(double k, double R) {
  const double x = k * R;
  return 3.0 / (x * x) * (c_sin(x) / x - c_cos(x));
}

static float sigma2_f(const float* k, const float* P, int Nk, float R) {
  float acc = 0.0f;
  for (int i = 0; i < Nk - 1; i++)
    acc += (k[i + 1] - k[i]) / 2.0 *
           (P[i] * c_pow(k[i] * tophat_f(k[i], R), 2) + P[i + 1] * c_pow(k[i + 1] * tophat_f(k[i + 1], R), 2));
  return (float)(acc / (2.0 * M_PI * M_PI));
}
static double sigma2_d(const float* k, const float* P, int Nk, double R) {
  double acc = 0.0;
  for (int i = 0; i < Nk - 1; i++) {
    const double k0 = k[i], k1 = k[i + 1];
    const double w0 = k0 * tophat_d(k0, R), w1 = k1 * tophat_d(k1, R);
    acc += (k1 - k0) / 2.0 * ((double)P[i] * w0 * w0 + (double)P[i + 1] * w1 * w1);
  }
  return acc / (2.0 * M_PI * M_PI);
}

// Tinker et al. (2008) multiplicity function at Delta = 300
static float tinker_f(float s) {
  const float B = 0.466f, d = 2.06f, e = 0.99f, f = 0.48f, g = 1.310f;
  return (float)(B * (c_pow(s / e, -d) + c_pow(s, -f)) * c_exp(-g / (s * s)));
}
static double tinker_d(double s) {
  const double B = 0.466, d = 2.06, e = 0.99, f = 0.48, g = 1.310;
  return B * (c_pow(s / e, -d) + c_pow(s, -f)) * c_exp(-g / (s * s));
}

float barrier(const BoxParams& b, float S) {
  if (b.DO_EB == 0) return b.dc;
  return (float)(c_sqrt(b.a) * b.dc * (1.0 + b.beta * c_pow(S / (b.a * b.dc * b.dc), b.alpha)));
}

int halo_tables(const BoxParams& b, const float* K, const float* P, int Nk, int prec64, std::vector<float>& Sig_grid,
                std::vector<float>& Btab, std::vector<double>& M, std::vector<double>& Int) {
  const int Nr = Nk, Nc = ncells(b);
  if (Nr < 3 || Nc < 2) return EXH_E_INVALID;
  M.assign(Nr, 0.0);
  Int.assign(Nr, 0.0);
  std::vector<double> sig(Nr), R(Nr);
  if (!prec64) {
    const float Rmin = (float)c_pow(b.Mcell * 0.9 * 3.0 / (4.0 * M_PI * b.rhomz), 1.0 / 3.0);
    const float Rmax = (float)c_pow(kMmax * 3.0 / (4.0 * M_PI * b.rhomz), 1.0 / 3.0);
    for (int i = 0; i < Nr; i++) {
      const float r = (float)c_pow(10, c_log10(Rmin) + i * (c_log10(Rmax) - c_log10(Rmin)) / (Nr - 1));
      R[i] = r;
      M[i] = (double)4.0 / 3.0 * M_PI * ((float)b.rhomz * c_pow(r, 3));
    }
    parallel_for(Nr, [&](int i) { sig[i] = (double)c_sqrt(sigma2_f(K, P, Nk, (float)R[i])); });
  } else {
    const double Rmin = c_pow((double)b.Mcell * 0.9 * 3.0 / (4.0 * M_PI * (double)b.rhomz), 1.0 / 3.0);
    const double Rmax = c_pow(kMmax * 3.0 / (4.0 * M_PI * (double)b.rhomz), 1.0 / 3.0);
    for (int i = 0; i < Nr; i++) {
      R[i] = c_pow(10.0, c_log10(Rmin) + i * (c_log10(Rmax) - c_log10(Rmin)) / (Nr - 1));
      M[i] = 4.0 / 3.0 * M_PI * (double)b.rhomz * c_pow(R[i], 3);
    }
    parallel_for(Nr, [&](int i) { sig[i] = c_sqrt(sigma2_d(K, P, Nk, R[i])); });
  }
  Spline s;
  if (s.init(M.data(), sig.data(), Nr) != EXH_OK) return EXH_E_INVALID;
  Sig_grid.assign(Nc, 0.f);
  Sig_grid[0] = 1e+30f;
  int st = 0;
  for (int i = 1; i < Nc; i++) Sig_grid[i] = (float)c_pow(s.eval((double)i * b.Mcell, &st), 2.0);
  if (st) return EXH_E_RANGE;
  for (int i = 1; i < Nr; i++) {
    if (!prec64) {
      const float r1 = (float)R[i], r0 = (float)R[i - 1];
      Int[i] = Int[i - 1] - (double)(c_log(sig[i]) - c_log(sig[i - 1])) / 2.0 *
                                (tinker_f((float)sig[i]) / c_pow(r1, 3.0) + tinker_f((float)sig[i - 1]) / c_pow(r0, 3.0));
    } else {
      Int[i] = Int[i - 1] - (c_log(sig[i]) - c_log(sig[i - 1])) / 2.0 *
                                (tinker_d(sig[i]) / c_pow(R[i], 3.0) + tinker_d(sig[i - 1]) / c_pow(R[i - 1], 3.0));
    }
    if (Int[i] == Int[i - 1]) Int[i] = Int[i - 1] * 1.000001;
  }
  Btab.assign(Nc, 0.f);
  for (int c = 0; c < Nc; c++) Btab[c] = barrier(b, Sig_grid[c]);
  return EXH_OK;
}

int ladder_tables(const BoxParams& b, const float* K, const float* P, int Nk, int n_radii, float R_max,
                  std::vector<float>& R, std::vector<float>& B) {
  if (n_radii < 1 || n_radii > 255 || !(R_max >= b.Lc)) return EXH_E_INVALID;
  R.assign(n_radii, 0.f);
  B.assign(n_radii, 0.f);
  // log-spaced radii from one cell to R_max; sigma^2(R) by the FP64 top-hat
  // trapezoid on the input table, barrier of find_halos.c:200-212 at sigma^2
  const double lo = std::log((double)b.Lc), hi = std::log((double)R_max);
  std::vector<double> s2(n_radii);
  parallel_for(n_radii, [&](int i) {
    const double r = n_radii > 1 ? std::exp(lo + (hi - lo) * i / (n_radii - 1)) : (double)b.Lc;
    R[i] = (float)r;
    s2[i] = sigma2_d(K, P, Nk, r);
  });
  for (int i = 0; i < n_radii; i++) B[i] = barrier(b, (float)s2[i]);
  return EXH_OK;
}

int amplitude_table(const BoxParams& b, const float* K, const float* P, int Nk, std::vector<float>& A) {
  if (b.nd[0] != b.nd[1] || b.nd[0] != b.nd[2]) return EXH_E_UNSUPPORTED;
  std::vector<double> kd(Nk), pd(Nk);
  for (int i = 0; i < Nk; i++) { kd[i] = K[i]; pd[i] = P[i]; }      // Inter_Power, density_grid.c:47-50
  Spline s;
  if (s.init(kd.data(), pd.data(), Nk) != EXH_OK) return EXH_E_INVALID;
  const int h = b.nd[0] / 2;
  const int nmax = 3 * h * h;
  const double kf = 2.0 * M_PI / ((double)b.Lc * b.nd[0]);
  A.assign(nmax + 1, 0.f);
  int st = 0;
  for (int n2 = 1; n2 <= nmax; n2++) {
    const double k = kf * c_sqrt((double)n2);
    A[n2] = (float)c_sqrt(s.eval(k, &st) / 2.0);
  }
  return st ? EXH_E_RANGE : EXH_OK;
}

const std::vector<int>& cells_in_spheres() {
  // built once per process (thread-safe local static initialisation)
  static const std::vector<int> tab = [] {
    std::vector<int> tab;
    const int lmax = 10000, t = 100;
    std::vector<long> hist(lmax, 0);
    for (int i = -t; i <= t; i++)
      for (int j = -t; j <= t; j++)
        for (int k = -t; k <= t; k++) {
          const long d = (long)i * i + (long)j * j + (long)k * k;
          if (d < lmax) hist[d]++;
        }
    long cum = 0;
    for (int l = 0; l < lmax; l++)
      if (hist[l]) { cum += hist[l]; tab.push_back((int)cum); }
    return tab;
  }();
  return tab;
}

}  // namespace exh
