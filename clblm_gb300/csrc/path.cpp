// path.cpp -- the line of sight through the layered atmosphere and the
// layers it crosses (host code of the library, binary64): calculatePath
// (clblm_AtmPath.f90:871-964) with
//   refractiveIndex      :977-1004    the refractivity of each profile level
//   standardPathGeometry :1010-1131   FSCGEO case 2A (:1391-1700), FNDHMN
//                                     (:1718-1847), REDUCE (:2215-2269)
//   rayTraceAndLayerPack :1135-1301   RFPATH (:2535-2781) with AMERGE
//                                     (:2794-2973) and ALAYER (:3000-3246),
//                                     then FPACK (:3279-3483)
//   densityOnPathLevel   :1306-1355
// and the refraction model FNDSHD/SCLHTD (:3606-3700), ANDEXD/RADRFD
// (:3489-3530), EXPINT (src/common/clblm_Util.f90:92-106).
//
// The work is a few thousand scalar steps per path (once per scene, not per
// spectral point), so it stays on the host; every expression keeps the
// reference's order of operations so the layer amounts the device OD kernels
// take are the reference's to the last bit of its arithmetic.  Compiled
// without floating-point contraction.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/clblm_gb300.h"

namespace {

constexpr double kPi = 3.1415926535898;  // PI as clblm_ConstParam.f90 writes it
const double kDeg = 180.0 / kPi;
const double kGcair = 1.0E-3 * 8.314472E+07 / 6.02214199E+23;  // GCAIR = 1e-3*GASCON/AVOGAD
constexpr double kDeltas = 5.0;                                 // DELTAS [km]
constexpr double kAlosmt = 2.6867775E+19;                       // ALOSMT
constexpr double kTol = 5.E-4;                                  // AMERGE's and calcCLBLMPaths' TOL [km]

struct PathError {
  int code;
  std::string msg;
};
[[noreturn]] void stop(int code, const std::string& msg) { throw PathError{code, msg}; }

// EXPINT: exponential interpolation, linear where an end is zero
double expint(double x1, double x2, double a) {
  if (x1 == 0.0 || x2 == 0.0) return x1 + (x2 - x1) * a;
  return x1 * std::pow(x2 / x1, a);
}

// The refractivity n - 1 between two levels as gamma * exp(-h / sh)
// (SCLHTD); sh = 0 when the two agree to 1e-5 (then n - 1 = gamma).
struct Refractivity {
  double sh = 0.0, gamma = 0.0;
  static Refractivity fit(double z1, double z2, double rf1_in, double rf2_in) {
    Refractivity r;
    const double rf1 = rf1_in + 1.0E-20, rf2 = rf2_in + 1.0E-20;
    const double ratio = rf1 / rf2;
    if (std::fabs(ratio - 1.0) < 1.0E-05) {
      r.sh = 0.0;
      r.gamma = rf1_in;
    } else {
      r.sh = (z2 - z1) / std::log(ratio);
      r.gamma = rf1 * std::pow(rf2 / rf1, -z1 / (z2 - z1));
    }
    return r;
  }
  double index(double h) const { return sh == 0.0 ? 1.0 + gamma : 1.0 + gamma * std::exp(-h / sh); }  // ANDEXD
  double radius(double h) const { return sh == 0.0 ? 1.0E36 : sh * (1.0 + std::exp(h / sh) / gamma); }  // RADRFD
};

// The profile as the ray tracer sees it: altitudes, pressures, temperatures,
// refractivities, densities [lev][mol].  `z` is AMERGE's working copy (it
// may snap levels onto the path's boundaries); the ray's refraction is
// looked up in it (FNDSHD).
struct Profile {
  int n = 0, nmol = 0;
  double re = 0.0;
  std::vector<double> z, p, t, rf, den;
  // FNDSHD: the fit of the profile interval that holds h (its upper level
  // the first at or above h, at least the second level)
  Refractivity at(double h) const {
    int i2 = n - 1;
    for (int i = 1; i < n; ++i)
      if (z[i] >= h) {
        i2 = i;
        break;
      }
    return Refractivity::fit(z[i2 - 1], z[i2], rf[i2 - 1], rf[i2]);
  }
  double crfrct(double h) const { return (re + h) * at(h).index(h); }  // FNDHMN's CRFRCT after FNDSHD(h)
};

struct Geometry {
  double h1, h2, angle, phi, hmin;
  int len;
};

// FNDHMN (ITER = 0): the tangent height and the zenith angle at h2.
// Returns false when the ray cannot reach h2 (the reference's IERROR = 2).
bool fndhmn(const Profile& pr, double h1, double angle, double* h2, int* len, double* hmin, double* phi) {
  const double cpath = pr.crfrct(h1) * std::sin(angle / kDeg);
  double ch2 = pr.crfrct(*h2);
  if (std::fabs(cpath / ch2) > 1.0) return false;
  if (angle <= 90.0) {
    *len = 0;
    *hmin = h1;
  } else if (h1 > *h2 && *len != 1) {
    *len = 0;
    *hmin = *h2;
  } else {
    *len = 1;
    const double cmin = pr.crfrct(0.0);
    if (cpath < cmin) {  // the tangent point would be below the ground
      *h2 = 0.0;
      *hmin = 0.0;
      *len = 0;
      ch2 = cmin;
    } else {  // Newton's method on (re + h) n(h) = cpath, 0.2 km secant steps
      const double dh = 0.2, eta = 5.0E-7;
      double ht = h1 * std::sin(angle / kDeg) + (std::sin(angle / kDeg) - 1.0) * pr.re;
      for (int it = 1;; ++it) {
        const double ct = pr.crfrct(ht);
        if (std::fabs((cpath - ct) / cpath) < eta) break;
        if (it > 15) stop(CLBLM_ERR_ARG, "FNDHMN: the tangent height did not converge in 15 iterations");
        const double ctp = pr.crfrct(ht - dh);
        const double deriv = (ct - ctp) / dh;
        ht = ht + (cpath - ct) / deriv;
      }
      *hmin = ht;
    }
  }
  *phi = std::asin(cpath / ch2) * kDeg;
  if (angle <= 90.0 || *len == 1) *phi = 180.0 - *phi;
  return true;
}

// FSCGEO case 2A (H1, H2, ANGLE given; RANGE = BETA = 0).  Returns 0, 1 for a
// geometry it rejects (IERROR = 1) or 2 when the ray cannot reach H2.
int fscgeo_2a(const Profile& pr, Geometry* g, double zmax) {
  if (g->h1 >= g->h2 && g->angle <= 90.0) return 1;
  if (g->h1 == 0.0 && g->angle > 90.0) return 1;
  const double h2_given = g->h2;
  const bool reached = fndhmn(pr, g->h1, g->angle, &g->h2, &g->len, &g->hmin, &g->phi);
  if (g->h2 != h2_given) return 1;  // the ray met the ground
  if (!reached) return 2;
  g->len = g->hmin < std::min(g->h1, g->h2) ? 1 : 0;
  if (g->hmin >= zmax) return 1;
  if (g->h1 > zmax || g->h2 > zmax) {  // REDUCE: ends above the profile moved down to its top
    const double cpath = pr.at(g->h1).index(g->h1) * (pr.re + g->h1) * std::sin(g->angle / kDeg);
    const double czmax = pr.at(zmax).index(zmax) * (pr.re + zmax);
    const double angmax = 180.0 - std::asin(cpath / czmax) * kDeg;
    if (g->h1 > zmax) {
      g->h1 = zmax;
      g->angle = angmax;
    }
    if (g->h2 > zmax) {
      g->h2 = zmax;
      g->phi = angmax;
    }
  }
  return 0;
}

// One level of the merged path (AMERGE's ZPTH, PP, TP, RFNDXP, DENP)
struct PathLevel {
  double z, p, t, rf;
};

// AMERGE's result
struct Merge {
  std::vector<double> zout;       // the output (RT) boundaries, bottom up
  std::vector<PathLevel> lev;     // the merged levels
  std::vector<double> den;        // [lev][mol]
  int ihmid = -1;                 // merged level at min(H1, H2) (0-based), -1 none
};

// AMERGE: the output boundaries are the RT boundaries between HMIN and the
// path's top with HMIN, min(H1, H2) (a tangent path) and max(H1, H2); the
// merged levels are the profile's with the output boundaries interpolated
// in (pressure and refractivity and densities exponentially, temperature
// linearly).  Altitudes within TOL are snapped together.
Merge amerge(Profile& pr, double* h1, double h2, double hmin, int len, const std::vector<double>& zb) {
  Merge m;
  const double hmax = std::max(*h1, h2);
  double hmid = std::min(*h1, h2);
  std::vector<double> zh{hmin};
  if (len == 0) {
    zh.push_back(hmax);
  } else {
    zh.push_back(hmid);
    if (std::fabs(*h1 - h2) < kTol) *h1 = h2;
    if (*h1 != h2) zh.push_back(hmax);
  }
  const int nb = (int)zb.size();
  m.zout.push_back(zh[0]);
  int ib = nb - 1;
  for (int i = 0; i < nb; ++i) {
    if (std::fabs(zb[i] - zh[0]) < kTol) zh[0] = zb[i];
    if (zb[i] > zh[0]) {
      ib = i;
      break;
    }
  }
  for (size_t ih = 1; ih < zh.size();) {
    if (ib < nb) {
      if (std::fabs(zb[ib] - zh[ih]) < kTol) zh[ih] = zb[ib];
      if (zb[ib] < zh[ih]) {
        m.zout.push_back(zb[ib++]);
        continue;
      }
      if (zb[ib] == zh[ih]) ++ib;
    }
    m.zout.push_back(zh[ih++]);
  }
  int im = 0;
  while (im < pr.n && !(pr.z[im] >= hmin)) ++im;
  if (im >= pr.n) stop(CLBLM_ERR_ARG, "AMERGE: the profile does not reach the path's lowest point");
  const size_t limit = (size_t)pr.n + (size_t)nb + 3;
  double& ztop = m.zout.back();
  size_t iout = 0;
  for (;;) {
    if (m.lev.size() >= limit) stop(CLBLM_ERR_ARG, "AMERGE: more merged levels than the profile and boundaries");
    const int ip = (int)m.lev.size();
    bool from_profile = im < pr.n;
    if (from_profile) {
      if (std::fabs(m.zout[iout] - pr.z[im]) < kTol) pr.z[im] = m.zout[iout];
      if (m.zout[iout] < pr.z[im]) from_profile = false;
    }
    double zp;
    if (from_profile) {
      if (m.zout[iout] == pr.z[im]) ++iout;
      zp = pr.z[im];
      m.lev.push_back({zp, pr.p[im], pr.t[im], pr.rf[im]});
      for (int k = 0; k < pr.nmol; ++k) m.den.push_back(pr.den[(size_t)im * pr.nmol + k]);
      ++im;
      if (std::fabs(zp - hmid) < kTol) hmid = zp;
      if (zp == hmid) m.ihmid = ip;
      if (std::fabs(zp - ztop) < kTol) ztop = zp;
    } else {
      // the interval below the next profile level (the top interval past
      // the profile's end; the reference reads one level beyond there)
      const int jm = std::min(std::max(im, 1), pr.n - 1);
      const double zo = m.zout[iout];
      const double a = (zo - pr.z[jm - 1]) / (pr.z[jm] - pr.z[jm - 1]);
      PathLevel L;
      L.z = zo;
      L.p = expint(pr.p[jm - 1], pr.p[jm], a);
      L.t = pr.t[jm - 1] + (pr.t[jm] - pr.t[jm - 1]) * a;
      L.rf = expint(pr.rf[jm - 1], pr.rf[jm], a);
      for (int k = 0; k < pr.nmol; ++k)
        m.den.push_back(expint(pr.den[(size_t)(jm - 1) * pr.nmol + k], pr.den[(size_t)jm * pr.nmol + k], a));
      if (std::fabs(L.z - hmid) < kTol) L.z = hmid;
      if (L.z == hmid) m.ihmid = ip;
      ++iout;
      if (std::fabs(L.z - ztop) < kTol) L.z = ztop;
      zp = L.z;
      m.lev.push_back(L);
    }
    if (zp == ztop) break;
  }
  return m;
}

// The integrals ALAYER accumulates over one merged layer
struct LayerSums {
  double s = 0.0, bend = 0.0;           // path length, bending
  double psum = 0.0, tsum = 0.0, rho = 0.0;  // integrals of p*rho, p/GCAIR, rho along the path
};

// The ray's direction where it enters a layer
struct RayState {
  double sinai, cosai;
};

// ALAYER (IAMT = 1): the ray from the merged level j to j + 1 in steps of
// at most DELTAS, Simpson's rule in x = -r cos(i) for the path length and
// the bending, exponential (or linear) profiles of pressure, air density
// and each absorber.  amt[k] receives the absorber columns.
LayerSums alayer(const Merge& m, int j, const Refractivity& rfit, double cpath, double re, RayState* ray,
                 double* amt, std::vector<double>& dena, std::vector<double>& denb, std::vector<double>& hden) {
  const double eps = 1.0E-5;
  const int nmol = (int)dena.size();
  const PathLevel& la = m.lev[j];
  const PathLevel& lb = m.lev[j + 1];
  const double* dj = &m.den[(size_t)j * nmol];
  const double* dj1 = &m.den[(size_t)(j + 1) * nmol];
  const double z1 = la.z, z2 = lb.z;
  double h1 = z1, r1 = re + h1;
  const double dhmin = kDeltas * kDeltas / (2.0 * r1);
  double sinai1 = ray->sinai, cosai1 = ray->cosai;
  double y1 = 0.0, y3 = 0.0;
  if ((1.0 - ray->sinai) < eps) {  // near the tangent point: y = 1 - cos(i), by its series
    const double c2 = cosai1 * cosai1;
    y1 = c2 / 2.0 + c2 * c2 / 8.0 + c2 * c2 * c2 * 3.0 / 48.0;
  }
  double x1 = -r1 * cosai1;
  double ratio1 = r1 / rfit.radius(h1);
  double dsdx1 = 1.0 / (1.0 - ratio1 * sinai1 * sinai1);
  double dbndx1 = dsdx1 * sinai1 * ratio1 / r1;
  LayerSums out;
  double pa = la.p, pb = lb.p;
  if (pb == pa) stop(CLBLM_ERR_ARG, "ALAYER: pressures in adjoining layers must differ");
  double rhoa = pa / (kGcair * la.t), rhob = pb / (kGcair * lb.t);
  const double dz = z2 - z1;
  const double hp = -dz / std::log(pb / pa);
  const double hrho = std::fabs(rhob / rhoa - 1.0) >= eps ? -dz / std::log(rhob / rhoa) : 1.0E30;
  for (int k = 0; k < nmol; ++k) {
    dena[k] = dj[k];
    denb[k] = dj1[k];
    if ((dena[k] == 0.0 || denb[k] == 0.0) || std::fabs(1.0 - dena[k] / denb[k]) <= eps) hden[k] = 0.0;
    else hden[k] = -dz / std::log(denb[k] / dena[k]);
  }
  for (;;) {
    double dh = -kDeltas * cosai1;
    if (dh < dhmin) dh = dhmin;
    double h3 = h1 + dh;
    if (h3 > z2) h3 = z2;
    dh = h3 - h1;
    const double r3 = re + h3;
    const double h2 = h1 + dh / 2.0;
    const double r2 = re + h2;
    const double sinai2 = cpath / (rfit.index(h2) * r2);
    const double sinai3 = cpath / (rfit.index(h3) * r3);
    const double ratio2 = r2 / rfit.radius(h2);
    const double ratio3 = r3 / rfit.radius(h3);
    double cosai3, x3, w1, w2, w3;
    if ((1.0 - sinai2) <= eps) {
      y3 = y1 + (sinai1 * (1.0 - ratio1) / r1 + 4.0 * sinai2 * (1.0 - ratio2) / r2 + sinai3 * (1.0 - ratio3) / r3) *
                    dh / 6.0;
      cosai3 = -std::sqrt(2.0 * y3 - y3 * y3);
      x3 = -r3 * cosai3;
      const double dx = x3 - x1;
      w1 = 0.5 * dx;
      w2 = 0.0;
      w3 = 0.5 * dx;
    } else {
      const double cosai2 = -std::sqrt(1.0 - sinai2 * sinai2);
      cosai3 = -std::sqrt(1.0 - sinai3 * sinai3);
      const double x2 = -r2 * cosai2;
      x3 = -r3 * cosai3;
      const double d31 = x3 - x1, d32 = x3 - x2, d21 = x2 - x1;
      if (d32 == 0.0 || d21 == 0.0) {
        w1 = 0.5 * d31;
        w2 = 0.0;
        w3 = 0.5 * d31;
      } else {
        w1 = (2.0 - d32 / d21) * d31 / 6.0;
        w2 = d31 * d31 * d31 / (d32 * d21 * 6.0);
        w3 = (2.0 - d21 / d32) * d31 / 6.0;
      }
    }
    const double dsdx2 = 1.0 / (1.0 - ratio2 * sinai2 * sinai2);
    const double dsdx3 = 1.0 / (1.0 - ratio3 * sinai3 * sinai3);
    const double dbndx2 = dsdx2 * sinai2 * ratio2 / r2;
    const double dbndx3 = dsdx3 * sinai3 * ratio3 / r3;
    const double ds = w1 * dsdx1 + w2 * dsdx2 + w3 * dsdx3;
    out.s = out.s + ds;
    out.bend = out.bend + (w1 * dbndx1 + w2 * dbndx2 + w3 * dbndx3);
    const double dsdz = ds / dh;
    pb = pa * std::exp(-dh / hp);
    rhob = rhoa * std::exp(-dh / hrho);
    if ((dh / hrho) >= eps) {
      out.psum = out.psum + dsdz * (hp / (1.0 + hp / hrho)) * (pa * rhoa - pb * rhob);
      out.tsum = out.tsum + dsdz * hp * (pa - pb) / kGcair;
      out.rho = out.rho + dsdz * hrho * (rhoa - rhob);
    } else {
      out.psum = out.psum + 0.5 * ds * (pa * rhoa + pb * rhob);
      out.tsum = out.tsum + 0.5 * ds * (pa + pb) / kGcair;
      out.rho = out.rho + 0.5 * ds * (rhoa + rhob);
    }
    for (int k = 0; k < nmol; ++k) {
      if (hden[k] == 0.0 || std::fabs(dh / hden[k]) < eps) {
        denb[k] = dj[k] + (dj1[k] - dj[k]) * (h3 - z1) / dz;
        amt[k] = amt[k] + 0.5 * (dena[k] + denb[k]) * ds * 1.0E5;
      } else {
        denb[k] = dj[k] * std::exp(-(h3 - z1) / hden[k]);
        amt[k] = amt[k] + dsdz * hden[k] * (dena[k] - denb[k]) * 1.0E5;
      }
    }
    pa = pb;
    rhoa = rhob;
    std::copy(denb.begin(), denb.end(), dena.begin());
    if (!(h3 < z2)) {
      ray->sinai = sinai3;
      ray->cosai = cosai3;
      return out;
    }
    h1 = h3;
    r1 = r3;
    sinai1 = sinai3;
    ratio1 = ratio3;
    y1 = y3;
    cosai1 = cosai3;
    x1 = x3;
    dsdx1 = dsdx3;
    dbndx1 = dbndx3;
  }
}

void run(const clblm_path_in_t& in, clblm_path_t* out) {
  const int nlev = in.nlev, nmol = in.nmol;
  Profile pr;
  pr.n = nlev;
  pr.nmol = nmol;
  pr.re = in.earth_radius;
  pr.z.assign(in.z, in.z + nlev);
  pr.p.assign(in.p, in.p + nlev);
  pr.t.assign(in.t, in.t + nlev);
  pr.den.assign(in.den, in.den + (size_t)nlev * nmol);
  // refractiveIndex (LOWTRAN's formula): n - 1 at v_refrac
  pr.rf.resize(nlev);
  const double xv = in.v_refrac;
  for (int i = 0; i < nlev; ++i) {
    const double denw = in.h2o >= 0 ? pr.den[(size_t)i * nmol + in.h2o] : 0.0;
    const double pph2o = denw * 1013.25 * pr.t[i] / (273.15 * kAlosmt);
    const double a = xv / 1.14E+5, b = xv / 6.24E+4, d = xv / 1.7E+4;
    pr.rf[i] = ((83.42 + (185.08 / (1.0 - a * a)) + (4.11 / (1.0 - b * b))) * (pr.p[i] * 288.15) /
                    (1013.25 * pr.t[i]) -
                (43.49 - d * d) * (pph2o / 1013.25)) *
               1.0E-06;
  }
  // standardPathGeometry
  const double zmax = pr.z[nlev - 1], zmin = pr.z[0];
  Geometry g{in.obs_alt, in.view_ang <= 90. ? zmax : zmin, in.view_ang, 0.0, 0.0, 0};
  int ierr = fscgeo_2a(pr, &g, zmax);
  if (ierr == 2) {  // the ray misses the bottom: the path goes back up to the top
    g.h1 = in.obs_alt;
    g.angle = in.view_ang;
    g.h2 = zmax;
    ierr = fscgeo_2a(pr, &g, zmax);
  }
  if (ierr != 0)
    stop(CLBLM_ERR_ARG, ierr == 2 ? "FSCGEO: the line of sight cannot reach the end of the path"
                                  : "FSCGEO: impossible path geometry");
  out->hobs = g.h1;
  out->hend = g.h2;
  out->angle = g.angle;
  out->phi = g.phi;
  out->hmin = g.hmin;
  out->len = g.len;

  // RFPATH: the merged levels, the ray's constant cpath = (re + h) n(h) sin(i)
  double h1 = g.h1;
  const double h2 = g.h2, hmin = g.hmin;
  const int len = g.len;
  const bool upward = h1 <= h2;
  const double ha = upward ? h1 : h2;
  const double angle_a = upward ? g.angle : g.phi;
  Merge m = amerge(pr, &h1, h2, hmin, len, std::vector<double>(in.z_rt, in.z_rt + in.nrt));
  const int nl_path = (int)m.lev.size() - 1;
  double cpath;
  if (len == 0) cpath = (pr.re + ha) * pr.at(ha).index(ha) * std::sin(angle_a / kDeg);
  else cpath = (pr.re + hmin) * pr.at(hmin).index(hmin);
  RayState ray;
  double theta;
  if (len == 1) {
    ray = {1.0, 0.0};
    theta = 90.0;
  } else {
    theta = angle_a;
    if (angle_a <= 45.0) ray = {std::sin(angle_a / kDeg), -std::cos(angle_a / kDeg)};
    else ray = {std::cos((90.0 - angle_a) / kDeg), -std::sin((90.0 - angle_a) / kDeg)};
  }
  std::vector<LayerSums> sums(nl_path);
  std::vector<double> amtp((size_t)std::max(nl_path, 0) * nmol, 0.0);
  std::vector<double> dena(nmol), denb(nmol), hden(nmol);
  double beta = 0.0, s = 0.0, bendng = 0.0, phi = g.phi;
  for (int j = 0; j < nl_path; ++j) {
    const Refractivity rfit = Refractivity::fit(m.lev[j].z, m.lev[j + 1].z, m.lev[j].rf, m.lev[j + 1].rf);
    sums[j] = alayer(m, j, rfit, cpath, pr.re, &ray, &amtp[(size_t)j * nmol], dena, denb, hden);
    const double dbend = sums[j].bend * kDeg;
    phi = std::asin(ray.sinai) * kDeg;
    const double dbeta = theta - phi + dbend;
    phi = 180.0 - phi;
    s = s + sums[j].s;
    bendng = bendng + dbend;
    beta = beta + dbeta;
    theta = 180.0 - phi;
    if (len == 1 && j + 1 == m.ihmid) {  // below the tangent point's end: traversed twice
      bendng = 2.0 * bendng;
      beta = 2.0 * beta;
      s = 2.0 * s;
    }
  }
  if (!upward) phi = angle_a;
  out->range = s;
  out->beta = beta;
  out->bendng = bendng;
  out->phi_end = phi;

  // FPACK: the merged layers summed into the output layers
  const double hmid = std::min(h1, h2);
  std::vector<double> amttot(nmol, 0.0);
  for (int i = 0; i < nl_path; ++i) {
    const double fac = (len == 1 && m.lev[i + 1].z <= hmid) ? 2.0 : 1.0;
    for (int k = 0; k < nmol; ++k) amttot[k] = amttot[k] + fac * amtp[(size_t)i * nmol + k];
  }
  const int nout = (int)m.zout.size() - 1;  // output layers before the zeroing cut
  std::vector<LayerSums> lay(nout);
  std::vector<double> amount((size_t)nout * nmol, 0.0);
  std::vector<double> pz(nout + 1), tz(nout + 1);
  pz[0] = m.lev[0].p;
  tz[0] = m.lev[0].t;
  int l = 0;
  for (int ip = 0; ip < nl_path; ++ip) {
    if (l >= nout) stop(CLBLM_ERR_ARG, "FPACK: merged levels and output boundaries disagree");
    lay[l].psum = lay[l].psum + sums[ip].psum;
    lay[l].tsum = lay[l].tsum + sums[ip].tsum;
    lay[l].rho = lay[l].rho + sums[ip].rho;
    lay[l].s = lay[l].s + sums[ip].s;
    for (int k = 0; k < nmol; ++k)
      amount[(size_t)l * nmol + k] = amount[(size_t)l * nmol + k] + amtp[(size_t)ip * nmol + k];
    if (m.lev[ip + 1].z == m.zout[l + 1]) {
      pz[l + 1] = m.lev[ip + 1].p;
      tz[l + 1] = m.lev[ip + 1].t;
      ++l;
    }
  }
  if (l != nout) stop(CLBLM_ERR_ARG, "FPACK: merged levels and output boundaries disagree");
  std::vector<double> amtcum(nmol, 0.0);
  std::vector<char> skip(nmol);
  for (int k = 0; k < nmol; ++k) skip[k] = amttot[k] == 0.0;
  std::vector<int> ipath(nout);
  int nlay = nout;
  for (int L = 0; L < nout; ++L) {
    if (len != 1) {
      if (h1 < h2) ipath[L] = 3;
      if (h1 > h2) ipath[L] = 1;
    } else {
      if (m.zout[L] < hmid) ipath[L] = 2;
      if (m.zout[L] >= hmid && h1 > h2) ipath[L] = 1;
      if (m.zout[L] >= hmid && h1 < h2) ipath[L] = 3;
    }
    // zeroAbsAmt: absorbers whose column is exhausted to 0.1% on an upward
    // path (O2 excepted) are zeroed; the path ends where all of them are
    int nzero = 0;
    const int nmol_max = (in.o2 >= 0 && skip[in.o2]) ? nmol - 1 : nmol;
    const double fac = ipath[L] == 2 ? 2.0 : 1.0;
    bool cut = false;
    for (int k = 0; k < nmol; ++k) {
      double& a = amount[(size_t)L * nmol + k];
      bool zero = false;
      if (in.zero_abs_amt == 1) {
        if (skip[k]) zero = true;
        else if (!(k == in.o2 || ipath[L] != 3) && !(((amttot[k] - amtcum[k]) / amttot[k]) > 0.001)) zero = true;
      }
      if (zero) {
        skip[k] = 1;
        a = 0.0;
        if (++nzero >= nmol_max) {
          cut = true;
          break;
        }
      }
      amtcum[k] = amtcum[k] + fac * a;
    }
    if (cut) {
      // the reference jumps out before LMAX is first set: a cut in the
      // first layer keeps every layer, the ones above not normalised
      if (L == 0) stop(CLBLM_ERR_ARG, "FPACK: zeroAbsAmt zeroes every absorber of the first layer");
      nlay = L;
      break;
    }
  }
  if (nlay > out->cap) {
    char buf[96];
    std::snprintf(buf, sizeof buf, "the path has %d layers, the output holds %d", nlay, out->cap);
    stop(CLBLM_ERR_CAPACITY, buf);
  }
  out->nlay = nlay;
  for (int L = 0; L <= nlay; ++L) {
    out->z[L] = m.zout[L];
    out->p[L] = pz[L];
    out->t[L] = tz[L];
  }
  for (int L = 0; L < nlay; ++L) {
    out->pave[L] = lay[L].psum / lay[L].rho;
    out->tave[L] = lay[L].tsum / lay[L].rho;
    out->wtot[L] = lay[L].rho * 1.0E+5;
    out->secant[L] = lay[L].s / (m.zout[L + 1] - m.zout[L]);
    out->ipath[L] = ipath[L];
    for (int k = 0; k < nmol; ++k) out->w[(size_t)L * nmol + k] = amount[(size_t)L * nmol + k];
  }
  if (out->q) {
    // densityOnPathLevel: the caller's profile (not AMERGE's snapped copy)
    // interpolated to the path's levels
    int lp = 1;
    for (int L = 0; L <= nlay; ++L) {
      const double zr = out->z[L];
      while (!(zr <= in.z[lp] || lp == nlev - 1)) ++lp;
      double a;
      if (std::fabs(zr - in.z[lp]) < kTol) a = 1.0;
      else if (std::fabs(zr - in.z[lp - 1]) < kTol) a = 0.0;
      else a = (zr - in.z[lp - 1]) / (in.z[lp] - in.z[lp - 1]);
      for (int k = 0; k < nmol; ++k)
        out->q[(size_t)L * nmol + k] = expint(in.den[(size_t)(lp - 1) * nmol + k], in.den[(size_t)lp * nmol + k], a);
    }
  }
}

}  // namespace

extern "C" int clblm_path(const clblm_path_in_t* in, clblm_path_t* out, char* errbuf, int32_t errlen) {
  auto fail = [&](int code, const std::string& msg) {
    if (errbuf && errlen > 0) std::snprintf(errbuf, (size_t)errlen, "%s", msg.c_str());
    return code;
  };
  if (!in || !out) return fail(CLBLM_ERR_ARG, "null argument");
  if (in->nlev < 2 || in->nmol < 0 || in->nrt < 2 || !in->z || !in->p || !in->t || (in->nmol > 0 && !in->den) ||
      !in->z_rt)
    return fail(CLBLM_ERR_ARG, "the profile needs 2 or more levels and the RT grid 2 or more boundaries");
  if (in->h2o >= in->nmol || in->o2 >= in->nmol) return fail(CLBLM_ERR_ARG, "h2o or o2 is not a column of den");
  if (!(in->earth_radius > 0.0)) return fail(CLBLM_ERR_ARG, "earth_radius must be positive");
  for (int i = 1; i < in->nlev; ++i)
    if (!(in->z[i] > in->z[i - 1])) return fail(CLBLM_ERR_ARG, "profile altitudes must ascend");
  for (int i = 1; i < in->nrt; ++i)
    if (!(in->z_rt[i] > in->z_rt[i - 1])) return fail(CLBLM_ERR_ARG, "RT boundaries must ascend");
  if (out->cap < 0 || (out->cap > 0 && (!out->z || !out->p || !out->t || !out->pave || !out->tave || !out->wtot ||
                                        (in->nmol > 0 && !out->w) || !out->secant || !out->ipath)))
    return fail(CLBLM_ERR_ARG, "null output array");
  try {
    run(*in, out);
  } catch (const PathError& e) {
    return fail(e.code, e.msg);
  } catch (const std::bad_alloc&) {
    return fail(CLBLM_ERR_ARG, "host allocation failed");
  }
  return CLBLM_OK;
}
