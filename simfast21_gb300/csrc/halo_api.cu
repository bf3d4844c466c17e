// C-ABI of the GPU excursion-set halo finder (include/sf21_halos.h).
//
// Host side: the per-redshift mass schedule in double precision with the
// reference's formulas and operation order (auxiliary.c: Eisenstein & Hu
// transfer function :28-210, sigma(R) by adaptive 15-point Gauss-Kronrod
// quadrature :366-424, Sheth-Tormen barrier :429-441, mass function
// :507-532, growth :224-266), the sphere of each mass as row runs (the
// offsets get_halos.c:244-257 visits), and the launch sequence:
//   once per density box: forward transform of delta_z0 (:127-138)
//   per redshift (:178-379):
//     filter bank: pairs of active masses per complex inverse transform,
//       thresholds -> one candidate bit set per mass        (:211-239)
//     per mass, in order: candidate list, prefilter against the flags of
//       larger masses, parallel rounds, sequential finisher, records
//                                                           (:240-282)
//     cell-size cycle                                       (:293-321)
//     subgrid cycle                                         (:326-371)
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <thread>
#include <vector>

#include "../../include/sf21_halos.h"
#include "sf21_kernels.h"

using namespace sf21;

namespace {

const double kPI = 3.1415926535897932385E0;  // Input_variables.h:10
const double kRHO0 = 2.775e11;               // Input_variables.h:11, Msun/h/(Mpc/h)^3
const double kH0 = 3.24078e-18;              // Input_variables.h:108, h/s

// ---- cosmology of auxiliary.c, host double --------------------------------
struct EH {  // what Set_Cosmology (:28-150) leaves for the transfer function
  double omhh, theta_cmb, alpha_gamma, sound_horizon_fit, beta_c, growth_to_z0;
};

EH eh_at(const sf21_halo_config& c, double redshift) {
  const double h = c.hubble, omm = c.omega_m, lamb = c.omega_lambda;
  const double omb = c.omega_b <= 0 ? 1e-5 : c.omega_b;
  EH e;
  e.theta_cmb = 2.728 / 2.7;
  const double omega_curv = 1.0 - omm - lamb;
  e.omhh = omm * (h * h);
  const double obhh = omb * (h * h);
  const double fb = omb / omm, fcdm = 1.0 - fb;
  const double th2 = e.theta_cmb * e.theta_cmb;
  const double z_eq = 25000.0 * e.omhh / (th2 * th2);
  const double b1 = 0.313 * pow(e.omhh, -0.419) * (1 + 0.607 * pow(e.omhh, 0.674));
  const double b2 = 0.238 * pow(e.omhh, 0.223);
  const double z_drag = 1291 * pow(e.omhh, 0.251) / (1.0 + 0.659 * pow(e.omhh, 0.828)) * (1.0 + b1 * pow(obhh, b2));
  const double y_drag = z_eq / (1.0 + z_drag);
  e.sound_horizon_fit = 44.5 * log(9.83 / e.omhh) / sqrt(1.0 + 10.0 * pow(obhh, 0.75));
  const double p_c = 0.25 * (5.0 - sqrt(1 + 24.0 * fcdm));
  const double zp = 1.0 + redshift;
  const double den = lamb + (zp * zp) * (omega_curv + omm * zp);
  const double olz = lamb / den, omz = omm * (zp * zp) * zp / den;
  const double g_k0 = z_eq / zp * 2.5 * omz / (pow(omz, 4.0 / 7.0) - olz + (1.0 + omz / 2.0) * (1.0 + olz / 70.0));
  const double g_0 = z_eq * 2.5 * omm / (pow(omm, 4.0 / 7.0) - lamb + (1.0 + omm / 2.0) * (1.0 + lamb / 70.0));
  e.growth_to_z0 = g_k0 / g_0;
  const double alpha_nu = (1 - fb) * (5 - 2 * p_c) / (5) * pow(1 + y_drag, -p_c) *
                          (1 + fb * (-0.553 + 0.126 * fb * fb)) *
                          (1 + (p_c) / 2 * (1 + 1 / (3. - 4. * p_c) / (7.)) / (1 + y_drag));
  e.alpha_gamma = sqrt(alpha_nu);
  e.beta_c = 1 / (1 - 0.949 * fb);
  return e;
}

double eh_tf(double kk, const EH& e) {  // :154-207, kk in 1/Mpc
  const double qq = kk / e.omhh * (e.theta_cmb * e.theta_cmb);
  const double x = kk * e.sound_horizon_fit * 0.43;
  const double x2 = x * x;
  const double gamma_eff = e.omhh * (e.alpha_gamma + (1 - e.alpha_gamma) / (1 + x2 * x2));
  const double qe = qq * e.omhh / gamma_eff;
  const double tl = log(2.71828 + 1.84 * e.beta_c * e.alpha_gamma * qe);
  const double tc = 14.4 + 325 / (1 + 60.5 * pow(qe, 1.11));
  return tl / (tl + tc * (qe * qe));
}

struct SigmaArgs {
  const sf21_halo_config* c;
  EH e;
  double R;
};

double pk_z0(double k, const SigmaArgs& s) {  // powerFunction :316-330, k in h/Mpc
  const double dH = 4.2E-5;
  const double t = eh_tf(k * s.c->hubble, s.e);
  return s.e.growth_to_z0 * s.e.growth_to_z0 *
         (pow((1 / k), 3) * 2 * pow(kPI * dH, 2) * pow((k * s.c->hubble), s.c->n_index + 3) * pow(t, 2));
}

double j1x(double x) { return x < 0.03 ? (1.0 / 3.0 - x * x * 1.0 / 30.0) : -(cos(x) - (sin(x) / x)) / x / x; }

double sigma_integrand(double x, const SigmaArgs& s) {  // dsigmaR :366-374
  const double R = s.R;
  const double w1 = 9.0 * j1x(x) * j1x(x), w2 = 9.0 * j1x(1 / x) * j1x(1 / x);
  return (pk_z0(x / R, s) / (2 * kPI * kPI) * (pow(x / R, 3)) * w1 / x +
          pk_z0(1 / x / R, s) / (2 * kPI * kPI) * (pow(1 / x / R, 3)) * w2 / x);
}

// Adaptive quadrature on [a, b] with the 15-point Gauss-Kronrod rule and
// bisection of the subinterval of largest error estimate (QUADPACK QAG,
// Piessens et al. 1983, the routine auxiliary.c:394-396 calls with
// epsabs 0, epsrel 3e-7, limit 1000).
struct GK15 {
  // Kronrod nodes (odd entries are the 7-point Gauss nodes), weights
  double x[8] = {0.991455371120812639206854697526329, 0.949107912342758524526189684047851,
                 0.864864423359769072789712788640926, 0.741531185599394439863864773280788,
                 0.586087235467691130294144845693013, 0.405845151377397166906606412076961,
                 0.207784955007898467600689403773245, 0.0};
  double wg[4] = {0.129484966168869693270611432679082, 0.279705391489276667901467771423780,
                  0.381830050505118944950369775488975, 0.417959183673469387755102040816327};
  double wk[8] = {0.022935322010529224963732008058970, 0.063092092629978553290700663189204,
                  0.104790010322250183839876322541518, 0.140653259715525918745189590510238,
                  0.169004726639267902826583426598550, 0.190350578064785409913256402421014,
                  0.204432940075298892414161999234649, 0.209482141084727828012999174891714};
};

struct Piece {
  double a, b, r, e;
};

template <class F>
Piece gk15(const F& f, double a, double b, double* rabs_out, double* rasc_out) {
  static const GK15 q;
  double f1v[7], f2v[7];
  const double c = 0.5 * (a + b), h = 0.5 * (b - a), ah = fabs(h);
  const double fc = f(c);
  double rg = fc * q.wg[3], rk = fc * q.wk[7];
  double ra = fabs(rk);
  for (int j = 0; j < 3; ++j) {
    const int jj = 2 * j + 1;
    const double d = h * q.x[jj];
    const double y1 = f(c - d), y2 = f(c + d), s = y1 + y2;
    f1v[jj] = y1;
    f2v[jj] = y2;
    rg += q.wg[j] * s;
    rk += q.wk[jj] * s;
    ra += q.wk[jj] * (fabs(y1) + fabs(y2));
  }
  for (int j = 0; j < 4; ++j) {
    const int jj = 2 * j;
    const double d = h * q.x[jj];
    const double y1 = f(c - d), y2 = f(c + d), s = y1 + y2;
    f1v[jj] = y1;
    f2v[jj] = y2;
    rk += q.wk[jj] * s;
    ra += q.wk[jj] * (fabs(y1) + fabs(y2));
  }
  const double mean = rk * 0.5;
  double rasc = q.wk[7] * fabs(fc - mean);
  for (int j = 0; j < 7; ++j) rasc += q.wk[j] * (fabs(f1v[j] - mean) + fabs(f2v[j] - mean));
  double err = (rk - rg) * h;
  rk *= h;
  ra *= ah;
  rasc *= ah;
  err = fabs(err);
  if (rasc != 0.0 && err != 0.0) {
    const double s = pow(200.0 * err / rasc, 1.5);
    err = s < 1.0 ? rasc * s : rasc;
  }
  if (ra > DBL_MIN / (50.0 * DBL_EPSILON) && 50.0 * DBL_EPSILON * ra > err) err = 50.0 * DBL_EPSILON * ra;
  *rabs_out = ra;
  *rasc_out = rasc;
  return {a, b, rk, err};
}

template <class F>
double qag15(const F& f, double a, double b, double epsrel, size_t limit) {
  double ra0, rasc0;
  std::vector<Piece> w;
  w.reserve(limit);
  w.push_back(gk15(f, a, b, &ra0, &rasc0));
  const double r0 = w[0].r, e0 = w[0].e;
  double tol = epsrel * fabs(r0);
  if (e0 <= 50.0 * DBL_EPSILON * ra0 && e0 > tol) return r0;
  if ((e0 <= tol && e0 != rasc0) || e0 == 0.0 || limit == 1) return r0;
  double area = r0, errsum = e0;
  int ro1 = 0, ro2 = 0;
  bool stop = false;
  size_t it = 1;
  do {
    size_t m = 0;
    for (size_t k = 1; k < w.size(); ++k)
      if (w[k].e > w[m].e) m = k;
    const Piece pm = w[m];
    const double mid = 0.5 * (pm.a + pm.b);
    double ra1, rasc1, ra2, rasc2;
    const Piece p1 = gk15(f, pm.a, mid, &ra1, &rasc1);
    const Piece p2 = gk15(f, mid, pm.b, &ra2, &rasc2);
    const double r12 = p1.r + p2.r, e12 = p1.e + p2.e;
    errsum += e12 - pm.e;
    area += r12 - pm.r;
    if (rasc1 != p1.e && rasc2 != p2.e) {
      if (fabs(pm.r - r12) <= 1.0e-5 * fabs(r12) && e12 >= 0.99 * pm.e) ++ro1;
      if (it >= 10 && e12 > pm.e) ++ro2;
    }
    tol = epsrel * fabs(area);
    if (errsum > tol) {
      if (ro1 >= 6 || ro2 >= 20) stop = true;
      const double tiny = (1.0 + 100.0 * DBL_EPSILON) * (fabs(mid) + 1000.0 * DBL_MIN);
      if (fabs(pm.a) <= tiny && fabs(pm.b) <= tiny) stop = true;
    }
    // the half with the larger error keeps slot m, the other is appended
    if (p2.e > p1.e) {
      w[m] = p2;
      w.push_back(p1);
    } else {
      w[m] = p1;
      w.push_back(p2);
    }
    ++it;
  } while (it < limit && !stop && errsum > tol);
  double sum = 0.0;
  for (const Piece& p : w) sum += p.r;
  return sum;
}

double sigma_R(const sf21_halo_config& c, double R) {  // sigmaR :377-398
  SigmaArgs s{&c, eh_at(c, 0.0), R};
  const double v = qag15([&](double x) { return sigma_integrand(x, s); }, 0., 1., 3e-7, 1000);
  return sqrt(v);
}

struct Cosmo {
  const sf21_halo_config& c;
  double sig8_old;
  explicit Cosmo(const sf21_halo_config& cc) : c(cc), sig8_old(sigma_R(cc, 8.0)) {}
  double sigma(double R) const { return c.sigma8 / sig8_old * sigma_R(c, R); }  // :415-424
  double Hz(double z) const {                                                    // :224-226
    return c.hubble * kH0 * sqrt(c.omega_m * (1. + z) * (1. + z) * (1. + z) + c.omega_lambda);
  }
  double int_growth(double zz) const {  // :242-257
    const double dz = 0.001;
    double intg = 0., z;
    const double hz0 = Hz(0.);
    for (z = zz + dz / 2.; z < zz + 100.; z += dz) {
      const double hub = Hz(z) / hz0;
      intg += (1. + z) / hub / hub / hub;
    }
    return intg * dz;
  }
  double growth(double z) const { return Hz(z) / Hz(0) * int_growth(z) / int_growth(0.); }  // :262-266
  double rho_m() const { return c.omega_m * kRHO0 / c.hubble; }                               // Input_variables.c:119
  double mass_to_radius(double M) const {                                                      // :498-500
    return pow(3 * M / (4 * kPI * c.omega_m * kRHO0 / c.hubble), 1.0 / 3.0);
  }
  double delta_filter(double sg, double growth) const {  // :429-441
    const double dz = c.delta_c / growth;
    return sqrt(c.STa) * dz * (1.0 + c.STb * pow((sg * sg / (c.STa * dz * dz)), c.STc));
  }
  double mass_function(double z, double M, double growth) const {  // :507-532 (growth = getGrowth(z))
    const double M2 = M + (M / 1000.);
    const double a = 0.73, A = 0.353, p = 0.175, E = 2.71828182846;
    const double sM = sigma(mass_to_radius(M)) * growth;
    const double sMdm = sigma(mass_to_radius(M2)) * growth;
    const double dlnsdm = (sMdm - sM) / (M / 1000.);
    const double nu = sqrt(a) * c.delta_c / sM;
    (void)z;
    return (-c.omega_m * kRHO0 / c.hubble) / M * dlnsdm / sM * sqrt(2.0 / kPI) * A * (1 + pow(nu, -2 * p)) * nu *
           pow(E, -nu * nu / 2.0);
  }
  double bias(double sigmaM, double growth) const {  // :446-458
    sigmaM = sigmaM * growth;
    const double nu = c.delta_c / sigmaM;
    return (1.0 + ((nu * nu - 1.0) / c.delta_c)) * pow((1.0 + (1 / (2.0 * pow(nu, 4)))), 0.06 - 0.02 * c.n_index);
  }
};

// largest float <= d (a float v satisfies v > d  <=>  v > this)
float float_floor(double d) {
  float f = (float)d;
  if ((double)f > d) f = nextafterf(f, -INFINITY);
  return f;
}

// smallest float v with (double)v * g > d, for g > 0 (the predicate is
// monotone in v): binary search over the ordered float bit patterns
float float_threshold_mul(double g, double d) {
  // ordered key k in [-inf, +inf]: k >= 0 -> the float with bits k, k < 0 ->
  // the negative float with magnitude bits -k
  auto key_to_float = [](int64_t k) {
    const uint32_t u = k >= 0 ? (uint32_t)k : ((uint32_t)(-k) | 0x80000000u);
    float f;
    memcpy(&f, &u, 4);
    return f;
  };
  const int64_t lo0 = -(int64_t)0x7f800000, hi0 = (int64_t)0x7f800000;
  auto pred = [&](int64_t k) { return (double)key_to_float(k) * g > d; };
  if (!pred(hi0)) return INFINITY;
  if (pred(lo0)) return -INFINITY;
  int64_t lo = lo0, hi = hi0;  // pred(lo) false, pred(hi) true
  while (hi - lo > 1) {
    const int64_t mid = lo + (hi - lo) / 2;
    if (pred(mid))
      hi = mid;
    else
      lo = mid;
  }
  return key_to_float(hi);
}

struct MassPlan {
  sf21_halo_mass m;
  float thr = 0.f;
  std::vector<int4> runs, druns;  // sphere rows; D = S + S rows (rounds only)
  bool rounds = false;
  int runs_off = 0, druns_off = 0;  // offsets in the device tables
};

// Sphere rows of radius R (the offsets :244-257 visits): for every (di, dj)
// with di^2 dx^2 + dj^2 dx^2 <= R^2, the largest m with the row's p offsets
// -m..m inside, all in the reference's double arithmetic.
void sphere_runs(double R, double dx, long nc, std::vector<int4>& out) {
  out.clear();
  const double R2 = R * R;
  for (long ii = -nc; ii <= nc; ++ii) {
    const double x2 = ii * ii * dx * dx;
    for (long jj = -nc; jj <= nc; ++jj) {
      const double y2 = jj * jj * dx * dx;
      if (!(x2 + y2 <= R2)) continue;
      long m = 0;
      while (m + 1 <= nc) {
        const long pp = m + 1;
        const double z2 = pp * dx * pp * dx;
        if (x2 + y2 + z2 <= R2) ++m; else break;
      }
      out.push_back(make_int4((int)ii, (int)jj, (int)m, 0));
    }
  }
}

// D = S + S as rows: half-width max over row splits of m1 + m2
void sum_runs(const std::vector<int4>& S, long nc, std::vector<int4>& out) {
  const long w = 4 * nc + 1;
  std::vector<int> md((size_t)w * w, -1);
  for (const int4& a : S)
    for (const int4& b : S) {
      const long di = a.x + b.x + 2 * nc, dj = a.y + b.y + 2 * nc;
      int& v = md[(size_t)di * w + dj];
      v = std::max(v, a.z + b.z);
    }
  out.clear();
  for (long di = 0; di < w; ++di)
    for (long dj = 0; dj < w; ++dj) {
      const int v = md[(size_t)di * w + dj];
      if (v >= 0) out.push_back(make_int4((int)(di - 2 * nc), (int)(dj - 2 * nc), v, 0));
    }
}

constexpr long kRoundsMaxNc = 24;  // D tables for spheres up to this half-width
constexpr int kMaxRounds = 96;

// f(0), ..., f(n - 1) on the host's cores (the scalar work of a schedule is
// about a hundred independent adaptive integrations); each f(i) is the same
// arithmetic as a serial call, so the results do not depend on the split.
template <class F>
void host_parallel_for(int n, const F& f) {
  const unsigned hw = std::thread::hardware_concurrency();
  const int nt = std::max(1, std::min(n, (int)(hw ? hw : 1)));
  if (nt <= 1) {
    for (int i = 0; i < n; ++i) f(i);
    return;
  }
  std::vector<std::thread> th;
  for (int t = 0; t < nt; ++t)
    th.emplace_back([&, t] {
      for (int i = t; i < n; i += nt) f(i);
    });
  for (std::thread& x : th) x.join();
}

int plan_masses(const Cosmo& cs, double z, double growth, std::vector<sf21_halo_mass>& out) {
  const sf21_halo_config& c = cs.c;
  const double rhom = cs.rho_m(), dx = c.L / c.N_halo, L3 = c.L * c.L * c.L;
  const double mass_dx = rhom * pow(dx, 3) * pow(10.0, c.halo_dlm);  // get_halos.c:159
  double R = c.L / 2.0;  // global_halo_Rmax (Input_variables.c:122)
  double M = (4.0 / 3.0) * kPI * rhom * pow(R, 3);
  out.clear();
  while (M > mass_dx && M >= c.halo_Mmin) {  // :197
    sf21_halo_mass h;
    memset(&h, 0, sizeof h);
    h.M = M;
    h.R = R;
    long nc = (long)(R / dx);
    if (nc == 0) nc = 1;
    h.nc = (int)nc;
    out.push_back(h);
    if (out.size() > 4096) return SF21_E_ARG;
    M = M / pow(10.0, c.halo_dlm);  // :285-286
    R = pow(3 / 4.0 / kPI / rhom * M, 1.0 / 3);
  }
  // expected counts (:201) and, for the masses that pass the gate, the barrier (:204-205)
  host_parallel_for((int)out.size(), [&](int i) {
    sf21_halo_mass& h = out[i];
    h.dndm = cs.mass_function(z, h.M, growth) * h.M * (pow(10.0, c.halo_dlm) - 1) * L3;
    h.active = h.dndm > -log(1 - 0.1);
    h.dcmz = h.active ? growth * cs.delta_filter(cs.sigma(h.R), growth) : 0.0;
  });
  return SF21_OK;
}

bool config_ok(const sf21_halo_config* c, std::string* why) {
  if (!c) return (*why = "null config"), false;
  const long N = c->N_halo;
  const bool pow2 = N >= 16 && N <= 1024 && !(N & (N - 1));
  if (!pow2 && !gen_supported((int)N))
    return (*why = "N_halo must be a power of two in [16, 1024] or a product of 2, 3 and 5 with 8 | N, 24..1280"),
           false;
  if (!(c->L > 0) || !(c->hubble > 0) || !(c->omega_m > 0) || !(c->sigma8 > 0) || !(c->halo_dlm > 0) ||
      !(c->delta_c > 0) || !(c->STa > 0))
    return (*why = "need L, hubble, omega_m, sigma8, halo_dlm, critical_overdensity, STa > 0"), false;
  return true;
}

std::string g_halo_err;

}  // namespace

struct sf21_halo_ctx {
  sf21_halo_config cfg;
  int device = 0;
  long N = 0, n3 = 0, nwords = 0;
  double dx = 0, dk = 0;
  cudaStream_t stream = nullptr;
  float2 *d_tw = nullptr, *d_spec = nullptr, *d_work = nullptr;
  int KP = 2;  // mass pairs per filter-bank pass
  bool gen = false;  // side not a power of two: the shared-memory transforms (kernels_gen.cu)
  GenPlan gp = {};
  float* d_delta = nullptr;
  bool have_density = false;
  uint32_t *d_FL = nullptr, *d_UND = nullptr, *d_ACC = nullptr, *d_bits = nullptr;
  std::vector<uint32_t*> d_masks;  // candidate bit sets, one per active mass of the last find
  std::vector<int> mask_of;        // schedule mass -> index in d_masks (-1 inactive)
  uint32_t *d_list = nullptr, *d_list2 = nullptr;
  uint8_t* d_status = nullptr;
  long list_cap = 0;
  uint32_t* d_chunk = nullptr;
  uint32_t* d_cnt = nullptr;   // [0] list length, [1] undecided, [2] second list length
  uint32_t* h_cnt = nullptr;   // pinned mirror
  float4* d_cat = nullptr;
  long cat_cap = 0, cat_n = 0;
  int4* d_runs = nullptr;
  long runs_cap = 0;
  std::vector<long> counts;
  std::vector<sf21_halo_mass> sched;
  uint32_t rng[3] = {0, 0, 0};
  // subgrid cycle (allocated / grown on use)
  uint32_t *d_sg_pow2 = nullptr, *d_sg_local = nullptr;
  uint8_t* d_sgL = nullptr;
  long sgL_cap = 0;
  uint8_t* d_sgX = nullptr;
  uint16_t* d_sgD = nullptr;
  uint32_t* d_sg_cnt = nullptr;
  uint32_t* d_sg_start = nullptr;  // taus state at each block's first position
  uint32_t* d_sgLB = nullptr;      // per block: bit set of the positions with draws of k >= 1
  SgEntryBufs sg_eb = {};
  long sg_blocks_cap = 0;
  uint64_t* d_sg_dn = nullptr;
  uint8_t* d_sg_dk = nullptr;
  uint32_t *d_sg_cell = nullptr, *d_sg_nn = nullptr;
  long sg_draw_cap = 0;
  uint32_t *d_sg_wpre = nullptr, *d_sg_chunk = nullptr;
  long sg_chunk_cap = 0;
  uint64_t* d_sg_u64 = nullptr;  // [0] positions consumed, [1] draws available
  int* d_sg_err = nullptr;
  std::string err;
};

#define HCTX_FAIL(ctx, code, ...)           \
  do {                                      \
    char _b[512];                           \
    snprintf(_b, sizeof(_b), __VA_ARGS__);  \
    (ctx)->err = _b;                        \
    return (code);                          \
  } while (0)

#define HCTX_CUDA(ctx, call)                                                                  \
  do {                                                                                        \
    cudaError_t _e = (call);                                                                  \
    if (_e != cudaSuccess)                                                                    \
      HCTX_FAIL(ctx, _e == cudaErrorMemoryAllocation ? SF21_E_ALLOC : SF21_E_CUDA, "%s failed: %s (%s:%d)", #call, \
                cudaGetErrorString(_e), __FILE__, __LINE__);                                 \
  } while (0)

static void taus_seed(uint32_t seed, uint32_t s[3]) {
  // gsl_rng_taus seeding (get_halos.c:70-71): seed 0 -> 1; three values of
  // the 69069 congruential sequence raised to each component's minimum;
  // six warm-up steps of the generator
  uint64_t x = seed ? seed : 1;
  uint32_t a = (uint32_t)((69069ull * x) & 0xffffffffull);
  if (a < 2) a += 2;
  uint32_t b = (uint32_t)((69069ull * a) & 0xffffffffull);
  if (b < 8) b += 8;
  uint32_t c = (uint32_t)((69069ull * b) & 0xffffffffull);
  if (c < 16) c += 16;
  for (int k = 0; k < 6; ++k) {
    a = ((a & 4294967294u) << 12) ^ (((a << 13) ^ a) >> 19);
    b = ((b & 4294967288u) << 4) ^ (((b << 2) ^ b) >> 25);
    c = ((c & 4294967280u) << 17) ^ (((c << 3) ^ c) >> 11);
  }
  s[0] = a;
  s[1] = b;
  s[2] = c;
}

// The generator's step T is linear over GF(2) in each 32-bit component:
// a jump by q steps is the matrix power T^q (column k = image of bit k).
struct TausMat {
  uint32_t col[3][32];
};

static uint32_t gf2_apply_h(const uint32_t* col, uint32_t v) {
  uint32_t r = 0;
  for (int k = 0; k < 32; ++k)
    if ((v >> k) & 1u) r ^= col[k];
  return r;
}

static TausMat taus_identity() {
  TausMat m;
  for (int c = 0; c < 3; ++c)
    for (int k = 0; k < 32; ++k) m.col[c][k] = 1u << k;
  return m;
}

static TausMat taus_one_step() {
  TausMat m;
  for (int k = 0; k < 32; ++k) {
    const uint32_t e = 1u << k;
    m.col[0][k] = ((e & 4294967294u) << 12) ^ (((e << 13) ^ e) >> 19);
    m.col[1][k] = ((e & 4294967288u) << 4) ^ (((e << 2) ^ e) >> 25);
    m.col[2][k] = ((e & 4294967280u) << 17) ^ (((e << 3) ^ e) >> 11);
  }
  return m;
}

static TausMat taus_mul(const TausMat& a, const TausMat& b) {  // a b
  TausMat r;
  for (int c = 0; c < 3; ++c)
    for (int k = 0; k < 32; ++k) r.col[c][k] = gf2_apply_h(a.col[c], b.col[c][k]);
  return r;
}

static void taus_jump(uint32_t s[3], uint64_t q) {
  TausMat p = taus_one_step();
  while (q) {
    if (q & 1)
      for (int c = 0; c < 3; ++c) s[c] = gf2_apply_h(p.col[c], s[c]);
    q >>= 1;
    if (q) p = taus_mul(p, p);
  }
}

static void free_hctx(sf21_halo_ctx* c) {
  if (!c) return;
  if (c->device >= 0) cudaSetDevice(c->device);
  void* ptrs[] = {c->d_tw,        c->d_spec,      c->d_work,      c->d_delta,     c->d_FL,        c->d_UND,
                  c->d_ACC,       c->d_bits,      c->d_list,      c->d_list2,     c->d_status,    c->d_chunk,
                  c->d_cnt,       c->d_cat,       c->d_runs,      c->d_sg_pow2,   c->d_sg_local,  c->d_sgL,
                  c->d_sgX,       c->d_sgD,       c->d_sg_cnt,    c->d_sg_start,  c->d_sgLB,      c->sg_eb.gx,    c->sg_eb.sx,    c->sg_eb.gentry,
                  c->sg_eb.sentry, c->sg_eb.bentry, c->sg_eb.gd,  c->sg_eb.sd,    c->sg_eb.gbase, c->sg_eb.sbase,
                  c->sg_eb.bbase, c->d_sg_dn,     c->d_sg_dk,     c->d_sg_cell,   c->d_sg_nn,     c->d_sg_wpre,
                  c->d_sg_chunk,  c->d_sg_u64,    c->d_sg_err};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (uint32_t* p : c->d_masks)
    if (p) cudaFree(p);
  if (c->h_cnt) cudaFreeHost(c->h_cnt);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

extern "C" int sf21_halo_schedule(const sf21_halo_config* cfg, double z, sf21_halo_mass* out, int cap) {
  std::string why;
  if (!config_ok(cfg, &why)) {
    g_halo_err = why;
    return -SF21_E_ARG;
  }
  std::vector<sf21_halo_mass> v;
  const Cosmo cs(*cfg);
  if (plan_masses(cs, z, cs.growth(z), v) != SF21_OK) {
    g_halo_err = "mass schedule longer than 4096 entries";
    return -SF21_E_ARG;
  }
  for (size_t k = 0; k < v.size() && (int)k < cap; ++k) out[k] = v[k];
  return (int)v.size();
}

extern "C" int sf21_halo_create(const sf21_halo_config* cfg, sf21_halo_ctx** out) {
  if (!out) return SF21_E_ARG;
  *out = nullptr;
  std::string why;
  if (!config_ok(cfg, &why)) {
    g_halo_err = why;
    return SF21_E_ARG;
  }
  sf21_halo_ctx* c = new sf21_halo_ctx();
  c->cfg = *cfg;
  c->device = cfg->device;
  c->N = cfg->N_halo;
  c->n3 = c->N * c->N * c->N;
  c->nwords = c->n3 / 32;
  c->dx = cfg->L / c->N;
  c->dk = 2 * kPI / cfg->L;
  taus_seed(0, c->rng);
#define HCREATE(call)                                                                       \
  do {                                                                                      \
    cudaError_t _e = (call);                                                                \
    if (_e != cudaSuccess) {                                                                \
      g_halo_err = std::string(#call) + " failed: " + cudaGetErrorString(_e);               \
      free_hctx(c);                                                                         \
      return _e == cudaErrorMemoryAllocation ? SF21_E_ALLOC : SF21_E_CUDA;                  \
    }                                                                                       \
  } while (0)
  const int N = (int)c->N;
  HCREATE(cudaSetDevice(c->device));
  HCREATE(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  c->gen = N & (N - 1);
  if (c->gen) {
    c->gp = gen_plan(N);
    HCREATE(gen_setup(N));
  } else {
    HCREATE(fft_setup(N));
    HCREATE(cb_setup(N));
    HCREATE(hf_setup(N));
  }
  const size_t box_c = sizeof(float2) * c->n3, bits = sizeof(uint32_t) * c->nwords;
  HCREATE(dev_malloc(&c->d_spec, box_c));
  HCREATE(dev_malloc(&c->d_work, box_c * c->KP));
  HCREATE(dev_malloc(&c->d_delta, sizeof(float) * c->n3));
  HCREATE(dev_malloc(&c->d_FL, bits));
  HCREATE(dev_malloc(&c->d_UND, bits));
  HCREATE(dev_malloc(&c->d_ACC, bits));
  HCREATE(dev_malloc(&c->d_bits, bits));
  HCREATE(cudaMemset(c->d_UND, 0, bits));
  HCREATE(cudaMemset(c->d_ACC, 0, bits));
  HCREATE(dev_malloc(&c->d_chunk, sizeof(uint32_t) * hf_compact_chunks(c->nwords)));
  HCREATE(dev_malloc(&c->d_cnt, sizeof(uint32_t) * 4));
  HCREATE(cudaMallocHost(&c->h_cnt, sizeof(uint32_t) * 4));
  std::vector<float2> tw(N);
  if (c->gen) {  // plain table exp(-2 pi i t / N)
    for (int t = 0; t < N; ++t) {
      const double ang = -2.0 * kPI * t / N;
      tw[t] = make_float2((float)cos(ang), (float)sin(ang));
    }
  } else {
    std::vector<double> tre(N), tim(N);
    twiddle_layout(N, tre.data(), tim.data());
    for (int t = 0; t < N; ++t) tw[t] = make_float2((float)tre[t], (float)tim[t]);
  }
  HCREATE(dev_malloc(&c->d_tw, sizeof(float2) * N));
  HCREATE(cudaMemcpy(c->d_tw, tw.data(), sizeof(float2) * N, cudaMemcpyHostToDevice));
#undef HCREATE
  *out = c;
  return SF21_OK;
}

extern "C" void sf21_halo_destroy(sf21_halo_ctx* c) { free_hctx(c); }

extern "C" const char* sf21_halo_last_error(const sf21_halo_ctx* c) {
  return c ? c->err.c_str() : g_halo_err.c_str();
}

static int set_density_dev(sf21_halo_ctx* c, const float* d, cudaStream_t st) {
  const int N = (int)c->N;
  Batch none;
  memset(&none, 0, sizeof(none));
  if (d != c->d_delta) HCTX_CUDA(c, cudaMemcpyAsync(c->d_delta, d, sizeof(float) * c->n3, cudaMemcpyDeviceToDevice, st));
  float2* packed = c->d_work;
  HCTX_CUDA(c, launch_t21_pack(c->n3, c->d_delta, packed, st));
  if (c->gen) {
    HCTX_CUDA(c, launch_gen_fwd_rows(c->gp, packed, c->d_spec, nullptr, c->d_tw, st));
    HCTX_CUDA(c, launch_gen_cols(c->gp, c->d_spec, none, 1, false, c->d_tw, st));
    HCTX_CUDA(c, launch_gen_cols(c->gp, c->d_spec, none, 0, false, c->d_tw, st));
  } else {
    HCTX_CUDA(c, launch_fwd_rows(N, packed, c->d_spec, nullptr, c->d_tw, st));
    HCTX_CUDA(c, launch_cols(N, c->d_spec, none, 1, 1, false, c->d_tw, st));
    HCTX_CUDA(c, launch_cols(N, c->d_spec, none, 1, 0, false, c->d_tw, st));
  }
  c->have_density = true;
  return SF21_OK;
}

extern "C" int sf21_halo_set_density(sf21_halo_ctx* c, const float* delta) {
  if (!c) return SF21_E_ARG;
  if (!delta) HCTX_FAIL(c, SF21_E_ARG, "null density box");
  HCTX_CUDA(c, cudaSetDevice(c->device));
  HCTX_CUDA(c, cudaMemcpyAsync(c->d_delta, delta, sizeof(float) * c->n3, cudaMemcpyHostToDevice, c->stream));
  const int rc = set_density_dev(c, c->d_delta, c->stream);
  if (rc) return rc;
  HCTX_CUDA(c, cudaStreamSynchronize(c->stream));
  return SF21_OK;
}

extern "C" int sf21_halo_set_density_device(sf21_halo_ctx* c, const float* d, void* stream) {
  if (!c) return SF21_E_ARG;
  if (!d) HCTX_FAIL(c, SF21_E_ARG, "null density box");
  HCTX_CUDA(c, cudaSetDevice(c->device));
  cudaStream_t st = stream ? (cudaStream_t)stream : c->stream;
  const int rc = set_density_dev(c, d, st);
  if (rc) return rc;
  if (st != c->stream) {  // later work on the context's stream sees the spectrum
    cudaEvent_t e;
    HCTX_CUDA(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    HCTX_CUDA(c, cudaEventRecord(e, st));
    HCTX_CUDA(c, cudaStreamWaitEvent(c->stream, e, 0));
    cudaEventDestroy(e);
  }
  return SF21_OK;
}

// read the counters (pinned) after the stream's work so far
static int read_counts(sf21_halo_ctx* c) {
  HCTX_CUDA(c, cudaMemcpyAsync(c->h_cnt, c->d_cnt, sizeof(uint32_t) * 4, cudaMemcpyDeviceToHost, c->stream));
  HCTX_CUDA(c, cudaStreamSynchronize(c->stream));
  return SF21_OK;
}

static int ensure_list(sf21_halo_ctx* c, long n) {
  if (n <= c->list_cap) return SF21_OK;
  long cap = std::max(n, std::max(2 * c->list_cap, (long)1 << 16));
  cap = std::min(cap, c->n3);
  if (c->d_list) cudaFree(c->d_list);
  if (c->d_list2) cudaFree(c->d_list2);
  if (c->d_status) cudaFree(c->d_status);
  c->d_list = c->d_list2 = nullptr;
  c->d_status = nullptr;
  c->list_cap = 0;
  HCTX_CUDA(c, dev_malloc(&c->d_list, sizeof(uint32_t) * cap));
  HCTX_CUDA(c, dev_malloc(&c->d_list2, sizeof(uint32_t) * cap));
  HCTX_CUDA(c, dev_malloc(&c->d_status, cap));
  c->list_cap = cap;
  return SF21_OK;
}

static int ensure_cat(sf21_halo_ctx* c, long n) {
  if (n <= c->cat_cap) return SF21_OK;
  const long cap = std::max(n, std::max(2 * c->cat_cap, (long)1 << 16));
  float4* p = nullptr;
  HCTX_CUDA(c, dev_malloc(&p, sizeof(float4) * cap));
  if (c->d_cat) {
    if (c->cat_n) HCTX_CUDA(c, cudaMemcpyAsync(p, c->d_cat, sizeof(float4) * c->cat_n, cudaMemcpyDeviceToDevice,
                                               c->stream));
    HCTX_CUDA(c, cudaStreamSynchronize(c->stream));
    cudaFree(c->d_cat);
  }
  c->d_cat = p;
  c->cat_cap = cap;
  return SF21_OK;
}

// sorted list of the set bits of W into list (slot 0) or list2 (slot 2);
// returns the count through *n
static int compact_bits(sf21_halo_ctx* c, const uint32_t* W, int slot, long* n) {
  cudaStream_t st = c->stream;
  const long nch = hf_compact_chunks(c->nwords);
  HCTX_CUDA(c, launch_bits_count(W, c->nwords, c->d_chunk, st));
  HCTX_CUDA(c, launch_scan_counts(c->d_chunk, nch, c->d_cnt + slot, st));
  int rc = read_counts(c);
  if (rc) return rc;
  *n = c->h_cnt[slot];
  if (*n == 0) return SF21_OK;
  if ((rc = ensure_list(c, *n))) return rc;
  HCTX_CUDA(c, launch_bits_emit(W, c->nwords, c->d_chunk, slot == 0 ? c->d_list : c->d_list2, st));
  return SF21_OK;
}

static int append_records(sf21_halo_ctx* c, const uint32_t* idx, long n, double M) {
  if (n <= 0) return SF21_OK;
  int rc = ensure_cat(c, c->cat_n + n);
  if (rc) return rc;
  HCTX_CUDA(c, launch_hf_records(idx, n, (int)c->N, (float)M, c->d_cat + c->cat_n, c->stream));
  c->cat_n += n;
  return SF21_OK;
}

// overlap test of one mass over its candidate bit set (get_halos.c:236-282)
static int greedy_mass(sf21_halo_ctx* c, const MassPlan& mp, const uint32_t* cand, long* found) {
  cudaStream_t st = c->stream;
  *found = 0;
  long n = 0;
  int rc = compact_bits(c, cand, 0, &n);
  if (rc) return rc;
  if (n == 0) return SF21_OK;
  const int4* runs = c->d_runs + mp.runs_off;
  const int nruns = (int)mp.runs.size();
  HCTX_CUDA(c, cudaMemsetAsync(c->d_cnt + 1, 0, sizeof(uint32_t), st));
  HCTX_CUDA(c, launch_hf_prefilter(c->d_list, c->d_cnt, (int)c->N, runs, nruns, c->d_FL, c->d_UND, c->d_status,
                                   c->d_cnt + 1, st));
  if ((rc = read_counts(c))) return rc;
  long und = c->h_cnt[1];
  if (und > 0 && mp.rounds) {
    const int4* druns = c->d_runs + mp.druns_off;
    const int nd = (int)mp.druns.size();
    int rounds = 0;
    while (und > 0 && rounds < kMaxRounds) {
      for (int k = 0; k < 4; ++k)
        HCTX_CUDA(c, launch_hf_round(c->d_list, c->d_cnt, (int)c->N, druns, nd, c->d_UND, c->d_ACC, c->d_status,
                                     c->d_cnt + 1, st));
      rounds += 4;
      if ((rc = read_counts(c))) return rc;
      und = c->h_cnt[1];
    }
  }
  HCTX_CUDA(c, launch_hf_flag_accepted(c->d_list, c->d_cnt, (int)c->N, runs, nruns, c->d_FL, c->d_status, st));
  if (und > 0)
    HCTX_CUDA(c, launch_hf_finisher(c->d_list, c->d_cnt, (int)c->N, runs, nruns, c->d_FL, c->d_ACC, c->d_status, st));
  long na = 0;
  if ((rc = compact_bits(c, c->d_ACC, 2, &na))) return rc;
  if ((rc = append_records(c, c->d_list2, na, mp.m.M))) return rc;
  HCTX_CUDA(c, launch_hf_clear(c->d_list, c->d_cnt, c->d_UND, c->d_ACC, st));
  *found = na;
  return SF21_OK;
}

template <class T>
static int grow(sf21_halo_ctx* c, T** p, long n, long* cap, bool keep_cap_var = false) {
  (void)keep_cap_var;
  if (n <= *cap && *p) return SF21_OK;
  if (*p) cudaFree(*p);
  *p = nullptr;
  HCTX_CUDA(c, dev_malloc(p, sizeof(T) * (size_t)std::max(n, 1L)));
  *cap = std::max(n, 1L);
  return SF21_OK;
}

static int sg_tables(sf21_halo_ctx* c) {
  if (c->d_sg_pow2) return SF21_OK;
  std::vector<uint32_t> p2((size_t)SG_POW2 * 96), loc((size_t)SG_LOCAL * 96);
  TausMat m = taus_one_step();
  for (int k = 0; k < SG_POW2; ++k) {
    for (int cc = 0; cc < 3; ++cc) memcpy(&p2[((size_t)k * 3 + cc) * 32], m.col[cc], 128);
    m = taus_mul(m, m);
  }
  const TausMat t1 = taus_one_step();
  const TausMat t4 = taus_mul(taus_mul(t1, t1), taus_mul(t1, t1));
  TausMat acc = taus_identity();
  for (int i = 0; i < SG_LOCAL; ++i) {  // column-major over i (see kernels_sg.cu)
    for (int cc = 0; cc < 3; ++cc)
      for (int k = 0; k < 32; ++k) loc[((size_t)cc * 32 + k) * SG_LOCAL + i] = acc.col[cc][k];
    acc = taus_mul(t4, acc);
  }
  HCTX_CUDA(c, dev_malloc(&c->d_sg_pow2, sizeof(uint32_t) * p2.size()));
  HCTX_CUDA(c, dev_malloc(&c->d_sg_local, sizeof(uint32_t) * loc.size()));
  HCTX_CUDA(c, cudaMemcpy(c->d_sg_pow2, p2.data(), sizeof(uint32_t) * p2.size(), cudaMemcpyHostToDevice));
  HCTX_CUDA(c, cudaMemcpy(c->d_sg_local, loc.data(), sizeof(uint32_t) * loc.size(), cudaMemcpyHostToDevice));
  HCTX_CUDA(c, dev_malloc(&c->d_sg_u64, sizeof(uint64_t) * 4));
  HCTX_CUDA(c, dev_malloc(&c->d_sg_err, sizeof(int) * 3));
  return SF21_OK;
}

static int sg_chunk(sf21_halo_ctx* c, long n) { return grow(c, &c->d_sg_chunk, scan_chunks(n), &c->sg_chunk_cap); }

// Subgrid cycle (get_halos.c:326-371) from the mass below the cell mass down
// to halo_Mmin; the context's generator continues across masses and calls.
static int subgrid_cycle(sf21_halo_ctx* c, const Cosmo& cs, double z, double growth, double M, long* total_out) {
  const sf21_halo_config& cf = c->cfg;
  cudaStream_t st = c->stream;
  *total_out = 0;
  if (!(M >= cf.halo_Mmin)) return SF21_OK;
  int rc = sg_tables(c);
  if (rc) return rc;
  const double rhom = cs.rho_m();
  double R = pow(3 / 4.0 / kPI / rhom * M, 1.0 / 3);
  // unflagged cells: per-word counts -> exclusive prefix (select by binary search)
  long wcap = c->nwords;
  if (!c->d_sg_wpre) HCTX_CUDA(c, dev_malloc(&c->d_sg_wpre, sizeof(uint32_t) * c->nwords));
  (void)wcap;
  if ((rc = sg_chunk(c, c->nwords))) return rc;
  HCTX_CUDA(c, launch_sg_free_count(c->d_FL, c->nwords, c->d_sg_wpre, st));
  HCTX_CUDA(c, launch_scan_u32(c->d_sg_wpre, c->nwords, c->d_sg_wpre, c->d_sg_chunk, c->d_cnt + 3, st));
  if ((rc = read_counts(c))) return rc;
  const uint64_t U = c->h_cnt[3];
  // the masses of the cycle (:329, :366-367) and their scalars (:332-334),
  // evaluated on the host cores in parallel
  struct SgMass {
    double M, dndm, hbias;
  };
  std::vector<SgMass> sm;
  for (double m = M, r = R; m >= cf.halo_Mmin;) {
    sm.push_back({m, r, 0.0});  // R parked in dndm until evaluated
    m = m / pow(10.0, cf.halo_dlm);
    r = pow(3 / 4.0 / kPI / rhom * m, 1.0 / 3);
  }
  host_parallel_for((int)sm.size(), [&](int i) {
    const double r = sm[i].dndm;
    const double sigma_aux = cs.sigma(r);
    sm[i].dndm = cs.mass_function(z, sm[i].M, growth) * sm[i].M * (pow(10.0, cf.halo_dlm) - 1) * pow(c->dx, 3);
    sm[i].hbias = cs.bias(sigma_aux, growth);
  });
  long total = 0;
  for (const SgMass& sgm : sm) {
    M = sgm.M;
    const double dndm = sgm.dndm, hbias = sgm.hbias;
    if (!(dndm <= 10.0))
      HCTX_FAIL(c, SF21_E_UNSUPPORTED, "subgrid: Poisson mean %g per cell above 10 (M = %E)", dndm, M);
    if (U > 0) {
      SgArgs a;
      memcpy(a.s0, c->rng, sizeof(a.s0));
      const double emu = exp(-dndm);
      const double xt = floor(ldexp(emu, 32));
      a.x1 = xt >= 4294967295.0 ? 0xffffffffu : (uint32_t)xt;
      memcpy(&a.emu, &emu, 8);
      // positions to generate: the mean consumption (1 + mu) per draw plus a margin
      const double need = (double)U * (1.0 + dndm) + 12.0 * sqrt((double)U * (1.0 + dndm) * (1.0 + dndm)) + 8 * SG_B;
      long nblocks = (long)ceil(need / SG_B);
      for (int attempt = 0;; ++attempt) {
        const long Q = nblocks * SG_B;
        if ((rc = grow(c, &c->d_sgL, Q, &c->sgL_cap))) return rc;
        if (nblocks > c->sg_blocks_cap || !c->d_sgX) {
          const long nb = nblocks, ng = sg_groups(nb), ns = sg_groups(ng);
          void* old[] = {c->d_sgX,        c->d_sgD,        c->d_sg_cnt,     c->d_sg_start,  c->d_sgLB,      c->sg_eb.gx,    c->sg_eb.sx,
                         c->sg_eb.gentry, c->sg_eb.sentry, c->sg_eb.bentry, c->sg_eb.gd,    c->sg_eb.sd,
                         c->sg_eb.gbase,  c->sg_eb.sbase,  c->sg_eb.bbase};
          for (void* q : old)
            if (q) cudaFree(q);
          c->d_sgX = nullptr;
          c->d_sgD = nullptr;
          c->d_sg_cnt = nullptr;
          c->d_sg_start = nullptr;
          c->d_sgLB = nullptr;
          c->sg_eb = SgEntryBufs{};
          c->sg_blocks_cap = 0;
          HCTX_CUDA(c, dev_malloc(&c->d_sgX, (size_t)nb * SG_LMAX));
          HCTX_CUDA(c, dev_malloc(&c->d_sgD, sizeof(uint16_t) * (size_t)nb * SG_LMAX));
          HCTX_CUDA(c, dev_malloc(&c->d_sg_cnt, sizeof(uint32_t) * (size_t)nb));
          HCTX_CUDA(c, dev_malloc(&c->d_sg_start, sizeof(uint32_t) * 3 * (size_t)nb));
          HCTX_CUDA(c, dev_malloc(&c->d_sgLB, sizeof(uint32_t) * (SG_B / 32) * (size_t)nb));
          HCTX_CUDA(c, dev_malloc(&c->sg_eb.gx, (size_t)ng * SG_LMAX));
          HCTX_CUDA(c, dev_malloc(&c->sg_eb.gd, sizeof(uint32_t) * (size_t)ng * SG_LMAX));
          HCTX_CUDA(c, dev_malloc(&c->sg_eb.sx, (size_t)ns * SG_LMAX));
          HCTX_CUDA(c, dev_malloc(&c->sg_eb.sd, sizeof(uint32_t) * (size_t)ns * SG_LMAX));
          HCTX_CUDA(c, dev_malloc(&c->sg_eb.sentry, (size_t)ns));
          HCTX_CUDA(c, dev_malloc(&c->sg_eb.sbase, sizeof(uint64_t) * (size_t)(ns + 1)));
          HCTX_CUDA(c, dev_malloc(&c->sg_eb.gentry, (size_t)ng));
          HCTX_CUDA(c, dev_malloc(&c->sg_eb.gbase, sizeof(uint64_t) * (size_t)ng));
          HCTX_CUDA(c, dev_malloc(&c->sg_eb.bentry, (size_t)nb));
          HCTX_CUDA(c, dev_malloc(&c->sg_eb.bbase, sizeof(uint64_t) * (size_t)nb));
          c->sg_blocks_cap = nb;
        }
        HCTX_CUDA(c, cudaMemsetAsync(c->d_sg_err, 0, sizeof(int) * 3, st));
        HCTX_CUDA(c, launch_sg_len(nblocks, a, c->d_sg_pow2, c->d_sg_local, c->d_sg_start, c->d_sgL, c->d_sgLB,
                                   c->d_sgX, c->d_sgD, c->d_sg_err, st));
        HCTX_CUDA(c, launch_sg_entries(c->d_sgX, c->d_sgD, nblocks, c->sg_eb, st));
        uint64_t avail = 0;
        int errf = 0;
        const long nsuper = sg_groups(sg_groups(nblocks));
        HCTX_CUDA(c, cudaMemcpyAsync(&avail, c->sg_eb.sbase + nsuper, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
        HCTX_CUDA(c, cudaMemcpyAsync(&errf, c->d_sg_err, sizeof(int), cudaMemcpyDeviceToHost, st));
        HCTX_CUDA(c, cudaStreamSynchronize(st));
        if (errf) HCTX_FAIL(c, SF21_E_UNSUPPORTED, "subgrid: a Poisson draw needed more than %d uniforms", SG_LMAX);
        if (avail >= U) break;
        if (attempt >= 3) HCTX_FAIL(c, SF21_E_ARG, "subgrid: stream positions short of the %llu draws",
                                    (unsigned long long)U);
        nblocks *= 2;
      }
      // draws with k >= 1: count per block, offsets, list
      HCTX_CUDA(c, launch_sg_walk(0, c->d_sgL, c->d_sgLB, nblocks, c->sg_eb.bentry, c->sg_eb.bbase, U, c->d_sg_cnt, c->d_sg_u64,
                                  nullptr, nullptr, 0, c->d_sg_err, st));
      if ((rc = sg_chunk(c, nblocks))) return rc;
      HCTX_CUDA(c, launch_scan_u32(c->d_sg_cnt, nblocks, c->d_sg_cnt, c->d_sg_chunk, c->d_cnt + 3, st));
      uint64_t consumed = 0;
      HCTX_CUDA(c, cudaMemcpyAsync(&consumed, c->d_sg_u64, sizeof(uint64_t), cudaMemcpyDeviceToHost, st));
      if ((rc = read_counts(c))) return rc;
      const long nd = c->h_cnt[3];
      long dcap = c->sg_draw_cap;
      if ((rc = grow(c, &c->d_sg_dn, nd, &dcap))) return rc;
      dcap = c->sg_draw_cap;
      if ((rc = grow(c, &c->d_sg_dk, nd, &dcap))) return rc;
      dcap = c->sg_draw_cap;
      if ((rc = grow(c, &c->d_sg_cell, nd, &dcap))) return rc;
      dcap = c->sg_draw_cap;
      if ((rc = grow(c, &c->d_sg_nn, nd, &dcap))) return rc;
      c->sg_draw_cap = std::max(c->sg_draw_cap, std::max(nd, 1L));
      long recs = 0;
      if (nd > 0) {
        HCTX_CUDA(c, launch_sg_walk(1, c->d_sgL, c->d_sgLB, nblocks, c->sg_eb.bentry, c->sg_eb.bbase, U, c->d_sg_cnt, nullptr,
                                    c->d_sg_dn, c->d_sg_dk, (uint64_t)c->sg_draw_cap, c->d_sg_err, st));
        uint64_t gb, hb;
        memcpy(&gb, &growth, 8);
        memcpy(&hb, &hbias, 8);
        HCTX_CUDA(c, launch_sg_nn(c->d_sg_dn, c->d_sg_dk, nd, c->d_FL, c->d_sg_wpre, c->nwords, c->d_delta, gb, hb,
                                  c->d_sg_cell, c->d_sg_nn, c->d_sg_err, st));
        if ((rc = sg_chunk(c, nd))) return rc;
        // offsets of the records in place of the per-draw indices (dn is no longer needed)
        uint32_t* off = reinterpret_cast<uint32_t*>(c->d_sg_dn);
        HCTX_CUDA(c, launch_scan_u32(c->d_sg_nn, nd, off, c->d_sg_chunk, c->d_cnt + 3, st));
        if ((rc = read_counts(c))) return rc;
        recs = c->h_cnt[3];
        if ((rc = ensure_cat(c, c->cat_n + recs))) return rc;
        HCTX_CUDA(c, launch_sg_records(c->d_sg_cell, c->d_sg_nn, off, nd, (int)c->N, (float)M, c->d_cat + c->cat_n,
                                       (uint64_t)(c->cat_cap - c->cat_n), c->d_sg_err, st));
        c->cat_n += recs;
      }
      int chk[3] = {0, 0, 0};
      HCTX_CUDA(c, cudaMemcpyAsync(chk, c->d_sg_err, sizeof(chk), cudaMemcpyDeviceToHost, st));
      HCTX_CUDA(c, cudaStreamSynchronize(st));
      if (chk[1])
        HCTX_FAIL(c, SF21_E_CUDA, "subgrid: access outside its buffer at site %d, index %d (skipped)", chk[1], chk[2]);
      taus_jump(c->rng, consumed);
      total += recs;
    }
  }
  *total_out = total;
  return SF21_OK;
}

static int run_filter_bank(sf21_halo_ctx* c, const std::vector<MassPlan>& plan, double growth) {
  const int N = (int)c->N;
  cudaStream_t st = c->stream;
  std::vector<int> act;
  for (size_t m = 0; m < plan.size(); ++m)
    if (plan[m].m.active) act.push_back((int)m);
  const float scale = (float)(c->dx * c->dx * c->dx / (c->cfg.L * c->cfg.L * c->cfg.L) * growth);
  size_t k0 = 0;
  while (k0 < act.size()) {
    HfBatch hb;
    memset(&hb, 0, sizeof(hb));
    hb.scale = scale;
    Batch bt;
    memset(&bt, 0, sizeof(bt));
    while (hb.K < c->KP && k0 < act.size()) {
      HfPair& p = hb.p[hb.K];
      const MassPlan& a = plan[act[k0]];
      p.dkRa = (float)(c->dk * a.m.R);
      p.thr_a = a.thr;
      p.bits_a = c->d_masks[c->mask_of[act[k0]]];
      if (k0 + 1 < act.size()) {
        const MassPlan& b = plan[act[k0 + 1]];
        p.dkRb = (float)(c->dk * b.m.R);
        p.thr_b = b.thr;
        p.bits_b = c->d_masks[c->mask_of[act[k0 + 1]]];
      }
      p.work = c->d_work + (size_t)hb.K * c->n3;
      bt.r[hb.K].work = p.work;
      k0 += p.bits_b ? 2 : 1;
      ++hb.K;
    }
    bt.K = hb.K;
    if (c->gen) {
      HCTX_CUDA(c, launch_gen_hf_rows_filter(c->gp, c->d_spec, hb, c->d_tw, st));
      HCTX_CUDA(c, launch_gen_hf_cols(c->gp, hb, 1, false, c->d_tw, st));
      HCTX_CUDA(c, launch_gen_hf_cols(c->gp, hb, 0, true, c->d_tw, st));
    } else {
      HCTX_CUDA(c, launch_hf_rows_filter_cb(N, c->d_spec, hb, c->d_tw, st));
      HCTX_CUDA(c, launch_cols_b_cb(N, bt, c->d_tw, st));
      HCTX_CUDA(c, launch_hf_cols_a_thresh_cb(N, hb, c->d_tw, st));
    }
  }
  return SF21_OK;
}

extern "C" int sf21_halo_find_z(sf21_halo_ctx* c, double z, long* nhalos) {
  if (!c) return SF21_E_ARG;
  if (!c->have_density) HCTX_FAIL(c, SF21_E_ARG, "no density box (sf21_halo_set_density first)");
  HCTX_CUDA(c, cudaSetDevice(c->device));
  cudaStream_t st = c->stream;
  const sf21_halo_config& cf = c->cfg;
  // schedule
  std::vector<sf21_halo_mass> ms;
  const Cosmo cs(cf);
  const double growth = cs.growth(z);
  if (plan_masses(cs, z, growth, ms) != SF21_OK) HCTX_FAIL(c, SF21_E_ARG, "mass schedule longer than 4096 entries");
  std::vector<MassPlan> plan(ms.size());
  std::vector<int4> table;
  c->mask_of.assign(ms.size(), -1);
  int nact = 0;
  for (size_t m = 0; m < ms.size(); ++m) {
    MassPlan& p = plan[m];
    p.m = ms[m];
    if (!p.m.active) continue;
    p.thr = float_floor(p.m.dcmz);
    sphere_runs(p.m.R, c->dx, p.m.nc, p.runs);
    p.rounds = p.m.nc <= kRoundsMaxNc && 4 * (long)p.m.nc + 1 <= c->N;
    if (p.rounds) sum_runs(p.runs, p.m.nc, p.druns);
    p.runs_off = (int)table.size();
    table.insert(table.end(), p.runs.begin(), p.runs.end());
    p.druns_off = (int)table.size();
    table.insert(table.end(), p.druns.begin(), p.druns.end());
    c->mask_of[m] = nact++;
  }
  if ((long)table.size() > c->runs_cap) {
    if (c->d_runs) cudaFree(c->d_runs);
    c->d_runs = nullptr;
    c->runs_cap = 0;
    HCTX_CUDA(c, dev_malloc(&c->d_runs, sizeof(int4) * std::max<size_t>(table.size(), 1)));
    c->runs_cap = (long)std::max<size_t>(table.size(), 1);
  }
  if (!table.empty())
    HCTX_CUDA(c, cudaMemcpyAsync(c->d_runs, table.data(), sizeof(int4) * table.size(), cudaMemcpyHostToDevice, st));
  while ((int)c->d_masks.size() < nact) {
    uint32_t* p = nullptr;
    HCTX_CUDA(c, dev_malloc(&p, sizeof(uint32_t) * c->nwords));
    c->d_masks.push_back(p);
  }
  // flags of this redshift (:181-182); the per-mass working sets start empty
  HCTX_CUDA(c, cudaMemsetAsync(c->d_FL, 0, sizeof(uint32_t) * c->nwords, st));
  HCTX_CUDA(c, cudaMemsetAsync(c->d_UND, 0, sizeof(uint32_t) * c->nwords, st));
  HCTX_CUDA(c, cudaMemsetAsync(c->d_ACC, 0, sizeof(uint32_t) * c->nwords, st));
  c->cat_n = 0;
  c->counts.assign(ms.size() + 2, 0);
  c->sched = ms;
  int rc = run_filter_bank(c, plan, growth);
  if (rc) return rc;
  for (size_t m = 0; m < ms.size(); ++m) {
    if (!plan[m].m.active) continue;
    long found = 0;
    if ((rc = greedy_mass(c, plan[m], c->d_masks[c->mask_of[m]], &found))) return rc;
    c->counts[m] = found;
  }
  // cell-size cycle (:293-321)
  const double rhom = cs.rho_m();
  double M = rhom * pow(c->dx, 3);
  if (M >= cf.halo_Mmin) {
    const double R = pow(3 / 4.0 / kPI / rhom * M, 1.0 / 3);
    const double dcell = growth * cs.delta_filter(cs.sigma(R), growth);
    const float tcell = float_threshold_mul(growth, dcell);
    HCTX_CUDA(c, launch_hf_cell(c->nwords, c->d_delta, tcell, c->d_FL, c->d_bits, st));
    long nc = 0;
    if ((rc = compact_bits(c, c->d_bits, 2, &nc))) return rc;
    if ((rc = append_records(c, c->d_list2, nc, M))) return rc;
    c->counts[ms.size()] = nc;
  }
  if (cf.use_subgrid == 1) {  // :323-371
    long nsg = 0;
    if ((rc = subgrid_cycle(c, cs, z, growth, M / pow(10.0, cf.halo_dlm), &nsg))) return rc;
    c->counts[ms.size() + 1] = nsg;
  }
  HCTX_CUDA(c, cudaStreamSynchronize(st));
  if (nhalos) *nhalos = c->cat_n;
  return SF21_OK;
}

extern "C" int sf21_halo_fetch(sf21_halo_ctx* c, sf21_halo_rec* out, long first, long count) {
  if (!c) return SF21_E_ARG;
  if (first < 0 || count < 0 || first + count > c->cat_n || (count && !out))
    HCTX_FAIL(c, SF21_E_ARG, "fetch range [%ld, %ld) outside the catalogue of %ld", first, first + count, c->cat_n);
  if (!count) return SF21_OK;
  HCTX_CUDA(c, cudaSetDevice(c->device));
  HCTX_CUDA(c, cudaMemcpyAsync(out, c->d_cat + first, sizeof(float4) * count, cudaMemcpyDeviceToHost, c->stream));
  HCTX_CUDA(c, cudaStreamSynchronize(c->stream));
  return SF21_OK;
}

extern "C" const sf21_halo_rec* sf21_halo_catalogue_device(const sf21_halo_ctx* c) {
  return c ? reinterpret_cast<const sf21_halo_rec*>(c->d_cat) : nullptr;
}

extern "C" int sf21_halo_counts(const sf21_halo_ctx* c, long* counts, int cap) {
  if (!c) return -SF21_E_ARG;
  for (size_t k = 0; k < c->counts.size() && (int)k < cap; ++k) counts[k] = c->counts[k];
  return (int)c->counts.size();
}

extern "C" int sf21_halo_rng_get(const sf21_halo_ctx* c, uint32_t state[3]) {
  if (!c || !state) return SF21_E_ARG;
  memcpy(state, c->rng, sizeof(c->rng));
  return SF21_OK;
}

extern "C" int sf21_halo_rng_set(sf21_halo_ctx* c, const uint32_t state[3]) {
  if (!c) return SF21_E_ARG;
  if (state)
    memcpy(c->rng, state, sizeof(c->rng));
  else
    taus_seed(0, c->rng);
  return SF21_OK;
}

extern "C" int sf21_halo_candidates(const sf21_halo_ctx* c0, int m, uint32_t* bits) {
  sf21_halo_ctx* c = const_cast<sf21_halo_ctx*>(c0);
  if (!c) return SF21_E_ARG;
  if (!bits || m < 0 || m >= (int)c->mask_of.size() || c->mask_of[m] < 0)
    HCTX_FAIL(c, SF21_E_ARG, "mass %d has no candidate set in the last find", m);
  HCTX_CUDA(c, cudaSetDevice(c->device));
  HCTX_CUDA(c, cudaMemcpyAsync(bits, c->d_masks[c->mask_of[m]], sizeof(uint32_t) * c->nwords,
                               cudaMemcpyDeviceToHost, c->stream));
  HCTX_CUDA(c, cudaStreamSynchronize(c->stream));
  return SF21_OK;
}

extern "C" int sf21_halo_field(sf21_halo_ctx* c, double z, int m, float* out) {
  if (!c) return SF21_E_ARG;
  if (!out) HCTX_FAIL(c, SF21_E_ARG, "null output");
  if (!c->have_density) HCTX_FAIL(c, SF21_E_ARG, "no density box (sf21_halo_set_density first)");
  std::vector<sf21_halo_mass> ms;
  const Cosmo cs0(c->cfg);
  if (plan_masses(cs0, z, cs0.growth(z), ms) != SF21_OK || m < 0 || m >= (int)ms.size())
    HCTX_FAIL(c, SF21_E_ARG, "mass %d not in the schedule", m);
  HCTX_CUDA(c, cudaSetDevice(c->device));
  const int N = (int)c->N;
  cudaStream_t st = c->stream;
  const Cosmo cs(c->cfg);
  HfBatch hb;
  memset(&hb, 0, sizeof(hb));
  hb.K = 1;
  hb.scale = (float)(c->dx * c->dx * c->dx / (c->cfg.L * c->cfg.L * c->cfg.L) * cs.growth(z));
  hb.p[0].dkRa = (float)(c->dk * ms[m].R);
  hb.p[0].work = c->d_work;
  hb.p[0].bits_a = c->d_bits;
  Batch bt;
  memset(&bt, 0, sizeof(bt));
  bt.K = 1;
  bt.r[0].work = c->d_work;
  Batch none;
  memset(&none, 0, sizeof(none));
  if (c->gen) {
    HCTX_CUDA(c, launch_gen_hf_rows_filter(c->gp, c->d_spec, hb, c->d_tw, st));
    HCTX_CUDA(c, launch_gen_cols(c->gp, c->d_work, none, 1, true, c->d_tw, st));
    HCTX_CUDA(c, launch_gen_cols(c->gp, c->d_work, none, 0, true, c->d_tw, st));
  } else {
    HCTX_CUDA(c, launch_hf_rows_filter(N, c->d_spec, hb, c->d_tw, st));
    HCTX_CUDA(c, launch_cols(N, nullptr, bt, 1, 1, true, c->d_tw, st));
    HCTX_CUDA(c, launch_cols(N, c->d_work, none, 1, 0, true, c->d_tw, st));
  }
  std::vector<float2> h(c->n3);
  HCTX_CUDA(c, cudaMemcpyAsync(h.data(), c->d_work, sizeof(float2) * c->n3, cudaMemcpyDeviceToHost, st));
  HCTX_CUDA(c, cudaStreamSynchronize(st));
  for (long t = 0; t < c->n3; ++t) out[t] = h[t].x;
  return SF21_OK;
}
