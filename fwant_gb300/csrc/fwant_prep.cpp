// fwant_prep: the input preprocessors of the solver stage as one program, a drop-in for the
// reference's seis3d_grid, seis3d_metric, seis3d_source and seis3d_station programs on one
// rank (code/srcF/seis3d_grid.F90, seis3d_metric.F90, seis3d_source.F90,
// seis3d_station.F90).  Each stage reads SeisFD3D.conf (ni, nj, nk, dims and the *_CONF /
// *_ROOT keys: para_init, grid_fnm_init, src_fnm_init, io_init) and writes the per-rank
// NetCDF file the solver imports:
//
//   fwant_prep grid    [SeisFD3D.conf]               GRID_CONF  -> GRID_ROOT/coord_mpi000000.nc
//   fwant_prep metric  [SeisFD3D.conf] [--device N]  coord      -> GRID_ROOT/metric_mpi000000.nc
//   fwant_prep source  [SeisFD3D.conf]               SOURCE_CONF + coord -> SOURCE_ROOT/source_mpi000000.nc
//   fwant_prep station [SeisFD3D.conf]               receivers of SeisFD3D.conf + coord
//                                                    -> STATION_ROOT/station_mpi000000.nc
//
// grid, source and station run on the host (a few thousand coordinates and a handful of
// points); metric evaluates the FP64 metric on the GPU (fwant_metric_arrays).  Every FP32
// expression is evaluated in the reference's order and precision (this file is compiled
// without contraction), so the files hold the values the reference's programs write.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>

#include "conf.h"
#include "fwant_gb300.h"
#include "netcdf3.h"

namespace {

constexpr double PI = 3.141592653589793;  // PI (mod_constants.F90:27)
constexpr float SEIS_ZERO = 1.0e-20f;      // SEIS_ZERO (mod_constants.F90:29)
constexpr int LENFD = 3;
const char* const SUFFIX = "mpi000000";

[[noreturn]] void die(const std::string& m) {
  std::fprintf(stderr, "fwant_prep: %s\n", m.c_str());
  std::exit(1);
}

// a real(SP) configuration value: the word rounded once to float, as a Fortran read does
float getf(const conf::Text& t, const std::string& key, int col) { return conf::to_float(t.get(key, col), t.path()); }

// real(SP) angle in degrees times PI / 180 in double, stored back in SP
// (pt_xyz(1:2,:)*PI/180.0_SP in io_pt_read, force_axis(1:2,n)*PI/180.0_SP in read_src_para)
float deg2rad_pt(float v) { return float(double(v) * PI / 180.0); }

struct Grid {
  int ni, nj, nk;
  int nx() const { return ni + 2 * LENFD; }
  int ny() const { return nj + 2 * LENFD; }
  int nz() const { return nk + 2 * LENFD; }
};

Grid main_grid(const conf::Text& cf) {
  Grid g{cf.get_int("ni", 2), cf.get_int("nj", 2), cf.get_int("nk", 2)};
  if (g.ni < 2 || g.nj < 2 || g.nk < 2) die(cf.path() + ": ni, nj and nk must be at least 2");
  if (cf.has("dims"))
    for (int d = 0; d < 3; ++d)
      if (cf.get_int("dims", d + 2) != 1) die("dims must be 1 1 1: one GPU runs the whole grid");
  return g;
}

std::vector<float> nc_floats(const nc3::Reader& f, const std::string& path, const std::string& name, size_t n) {
  std::vector<float> v;
  std::string err;
  if (!f.read(name, &v, &err)) die(path + ": " + err);
  if (v.size() != n) die(path + ": " + name + " has " + std::to_string(v.size()) + " values, expected " + std::to_string(n));
  return v;
}

struct Coord {
  std::vector<float> x, y, z;
};

// grid_coord_import (mod_grid.F90:96-103)
Coord read_coord(const conf::Text& cf, const Grid& g) {
  const std::string path = cf.get("GRID_ROOT", 2) + "/coord_" + SUFFIX + ".nc";
  nc3::Reader f;
  std::string err;
  if (!f.open(path, &err)) die(err);
  return {nc_floats(f, path, "x", g.nx()), nc_floats(f, path, "y", g.ny()), nc_floats(f, path, "z", g.nz())};
}

void write_or_die(const nc3::Writer& w, const std::string& path) {
  std::string err;
  if (!w.write(path, &err)) die(err);
}

// ---- grid: read_grid_coord (seis3d_grid.F90:89-149) and coord_skel (:151-176) -------------

// One axis with its ghosts.  A step of at least SEIS_ZERO gives the uniform axis
// (i - ni1)*dh + x0, or for z (k - num_z + LenFD)*dh + rmax so that the free surface sits at
// rmax; a smaller step reads the n interior values as one list-directed record after the
// anchor line ("<x", "<y", "<z").  theta and phi are degrees (gx/180.0_DP*PI), r is scaled by
// distance2meter; the ghosts are then extrapolated linearly from the interior edge.
std::vector<float> grid_axis(conf::Text& gc, int n, float dh, float x0, const char* anchor, bool top, bool degrees,
                             float d2m) {
  const int nxx = n + 2 * LENFD, i1 = LENFD, i2 = LENFD + n - 1;  // 0-based interior
  std::vector<float> g(nxx, 0.0f);
  if (dh >= SEIS_ZERO) {
    for (int q = 0; q < nxx; ++q) {
      const int idx = top ? q - nxx + 1 + LENFD : q - i1;
      g[q] = float(idx) * dh + x0;
    }
  } else {
    gc.seek(anchor);
    const std::vector<float> v = gc.record(size_t(n));
    for (int q = 0; q < n; ++q) g[i1 + q] = v[q];
  }
  for (float& v : g) v = degrees ? float(double(v) / 180.0 * PI) : v * d2m;
  for (int q = 1; q <= LENFD; ++q) {
    g[i1 - q] = (g[i1 - q + 1] + g[i1]) - g[i1 + 1];
    g[i2 + q] = (g[i2 + q - 1] + g[i2]) - g[i2 - 1];
  }
  return g;
}

void stage_grid(const conf::Text& cf) {
  const Grid g = main_grid(cf);
  conf::Text gc(cf.get("GRID_CONF", 2));
  const float d2m = getf(gc, "distance2meter", 2);
  float dh[3], x0[3];
  for (int d = 0; d < 3; ++d) {
    dh[d] = getf(gc, "steph", d + 2);
    x0[d] = getf(gc, "theta0_phi0_rmax", d + 2);
  }
  const std::vector<float> x = grid_axis(gc, g.ni, dh[0], x0[0], "<x", false, true, d2m);
  const std::vector<float> y = grid_axis(gc, g.nj, dh[1], x0[1], "<y", false, true, d2m);
  const std::vector<float> z = grid_axis(gc, g.nk, dh[2], x0[2], "<z", true, false, d2m);
  std::printf("output grid coordinate and locating ...\n");
  nc3::Writer w;
  const int dI = w.add_dim("I", g.nx()), dJ = w.add_dim("J", g.ny()), dK = w.add_dim("K", g.nz());
  w.add_var_f("x", {dI}, x.data(), x.size());
  w.add_var_f("y", {dJ}, y.data(), y.size());
  w.add_var_f("z", {dK}, z.data(), z.size());
  write_or_die(w, cf.get("GRID_ROOT", 2) + "/coord_" + SUFFIX + ".nc");
}

// ---- metric: seis3d_metric.F90:83-112 on the GPU, metric_skel (:132-160) ----------------

void stage_metric(const conf::Text& cf, int device) {
  const Grid g = main_grid(cf);
  const Coord c = read_coord(cf, g);
  std::vector<float> xsin(g.nx()), xcot(g.nx()), xi(g.nx()), eta(g.ny()), zeta(g.nz());
  const fwant_status rc = fwant_metric_arrays(g.ni, g.nj, g.nk, c.x.data(), c.y.data(), c.z.data(), device, xsin.data(),
                                              xcot.data(), xi.data(), eta.data(), zeta.data());
  if (rc != FWANT_OK) die("metric on the GPU failed (status " + std::to_string(int(rc)) + ")");
  std::printf("output metric ...\n");
  nc3::Writer w;
  const int dI = w.add_dim("I", g.nx()), dJ = w.add_dim("J", g.ny()), dK = w.add_dim("K", g.nz());
  w.add_var_f("xsin", {dI}, xsin.data(), xsin.size());
  w.add_var_f("xcot", {dI}, xcot.data(), xcot.size());
  w.add_var_f("xi_x", {dI}, xi.data(), xi.size());
  w.add_var_f("eta_y", {dJ}, eta.data(), eta.size());
  w.add_var_f("zeta_z", {dK}, zeta.data(), zeta.size());
  write_or_die(w, cf.get("GRID_ROOT", 2) + "/metric_" + SUFFIX + ".nc");
}

// minloc(abs(a - v)) as a 1-based index: the first of equal distances wins
int minloc_abs(const std::vector<float>& a, float v) {
  int best = 0;
  for (size_t q = 1; q < a.size(); ++q)
    if (std::fabs(a[q] - v) < std::fabs(a[best] - v)) best = int(q);
  return best + 1;
}

// ---- source: read_src_para (seis3d_source.F90:324-401), the locating loops (:60-160),
// ---- the distribution (:190-300) and srcnode_skel (:427-493) ----------------------------

// stf_name2id / stf_id2name (mod_src.F90:624-679)
struct StfName {
  const char* name;
  int id;
};
const StfName STF_NAMES[] = {{"gauss", 220}, {"gauss_int", 120}, {"ricker", 200}, {"bell", 230}, {"bell_int", 100},
                             {"triangle_int", 110}, {"B(shift)", 210}, {"step", 240}, {"delta", 250}};
int stf_name2id(const std::string& s) {
  for (const auto& e : STF_NAMES)
    if (s == e.name) return e.id;
  die("Have you told me how to generate the STF of " + s);
}

// angle2moment (seis3d_source.F90:403-425): the Aki & Richards moment tensor of a double
// couple in DP, rounded to SP, then turned to the spherical (theta, phi, r) components
void angle2moment(double strike, double dip, double rake, float m[6]) {
  const double dp = dip / 180.0 * PI, sp = strike / 180.0 * PI, rp = rake / 180.0 * PI;
  const double s1 = std::sin(sp), c1 = std::cos(sp);
  const float m11 = float(-(std::sin(dp) * std::cos(rp) * std::sin(2.0 * sp) + std::sin(2.0 * dp) * std::sin(rp) * (s1 * s1)));
  const float m22 = float(std::sin(dp) * std::cos(rp) * std::sin(2.0 * sp) - std::sin(2.0 * dp) * std::sin(rp) * (c1 * c1));
  const float m33 = -(m11 + m22);
  const float m12 = float(std::sin(dp) * std::cos(rp) * std::cos(2.0 * sp) +
                          0.5 * std::sin(2.0 * dp) * std::sin(rp) * std::sin(2.0 * sp));
  const float m13 = float(-(std::cos(dp) * std::cos(rp) * c1 + std::cos(2.0 * dp) * std::sin(rp) * s1));
  const float m23 = float(-(std::cos(dp) * std::cos(rp) * s1 - std::cos(2.0 * dp) * std::sin(rp) * c1));
  m[0] = m11; m[1] = m22; m[2] = m33;  // Mxx Myy Mzz
  m[3] = -m12; m[4] = m13; m[5] = -m23;  // Mxy Mxz Myz
}

struct Sources {
  int num = 0, ntw = 0, stf_id = 0;
  std::vector<float> time, freq;      // (ntw)
  std::vector<float> axis, t0;        // (3, num), (num)
  std::vector<float> val;             // (ntw, ncomp, num): Fx Fy Fz or Mxx Myy Mzz Mxy Mxz Myz
  std::vector<int> indx;              // (3, num)
  std::vector<float> shift;           // (3, num)
  std::vector<char> found;
};

// the key block of one source kind: number, window count, STF type and factors
void read_stf(conf::Text& sc, const char* kind, Sources& s) {
  const std::string k = kind;
  s.ntw = sc.get_int(k + "_stf_window", 2);
  if (s.ntw < 1) die(sc.path() + ": " + k + "_stf_window must be at least 1");
  s.stf_id = stf_name2id(sc.get(k + "_stf_type", 2));
  s.time.resize(s.ntw);
  s.freq.resize(s.ntw);
  for (int m = 0; m < s.ntw; ++m) {
    s.time[m] = getf(sc, k + "_stf_timefactor", m + 2);
    s.freq[m] = getf(sc, k + "_stf_freqfactor", m + 2);
  }
  s.axis.assign(size_t(3) * s.num, 0.0f);
  s.t0.assign(s.num, 0.0f);
  s.indx.assign(size_t(3) * s.num, 0);
  s.shift.assign(size_t(3) * s.num, 0.0f);
  s.found.assign(s.num, 0);
}

void read_forces(conf::Text& sc, Sources& f) {
  read_stf(sc, "force", f);
  f.val.assign(size_t(f.ntw) * 3 * f.num, 0.0f);
  sc.seek("<anchor_force>");
  for (int n = 0; n < f.num; ++n) {
    for (int m = 0; m < f.ntw; ++m) {
      const std::vector<float> r = sc.record(8);  // axis(3), t0, f0, Fx, Fy, Fz
      for (int d = 0; d < 3; ++d) f.axis[3 * n + d] = r[d];
      f.t0[n] = r[3];
      const float f0 = r[4];
      for (int c = 0; c < 3; ++c) f.val[(size_t(n) * 3 + c) * f.ntw + m] = r[5 + c] * f0;
    }
    for (int d = 0; d < 2; ++d) f.axis[3 * n + d] = deg2rad_pt(f.axis[3 * n + d]);
  }
}

void read_moments(conf::Text& sc, Sources& mo) {
  read_stf(sc, "moment", mo);
  mo.val.assign(size_t(mo.ntw) * 6 * mo.num, 0.0f);
  const std::string mech = sc.get("moment_mech_input", 2);
  sc.seek("<anchor_moment>");
  for (int n = 0; n < mo.num; ++n) {
    for (int m = 0; m < mo.ntw; ++m) {
      float t[6];
      float m0;
      if (mech == "moment") {
        const std::vector<float> r = sc.record(11);  // axis(3), t0, m0, Mxx Myy Mzz Mxy Mxz Myz
        for (int d = 0; d < 3; ++d) mo.axis[3 * n + d] = r[d];
        mo.t0[n] = r[3];
        m0 = r[4];
        for (int c = 0; c < 6; ++c) t[c] = r[5 + c];
      } else {
        // axis(3), t0, m0 in SP; strike, dip, rake in DP
        const std::vector<std::string> w = sc.words(8);
        for (int d = 0; d < 3; ++d) mo.axis[3 * n + d] = conf::to_float(w[d], sc.path());
        mo.t0[n] = conf::to_float(w[3], sc.path());
        m0 = conf::to_float(w[4], sc.path());
        angle2moment(conf::to_double(w[5], sc.path()), conf::to_double(w[6], sc.path()),
                     conf::to_double(w[7], sc.path()), t);
      }
      for (int c = 0; c < 6; ++c) mo.val[(size_t(n) * 6 + c) * mo.ntw + m] = m0 * t[c];
    }
    for (int d = 0; d < 2; ++d) mo.axis[3 * n + d] = deg2rad_pt(mo.axis[3 * n + d]);
  }
}

// fractional offset of the source from its node along one axis (1-based node i)
float node_shift(const std::vector<float>& a, int i, float v) {
  const float c = a[i - 1];
  return v > c ? (v - c) / (a[i] - c) : (v - c) / (c - a[i - 2]);
}

// nearest node and shift of every source inside this rank's domain
void locate_sources(Sources& s, const Coord& c, const Grid& g, float src_hyper_height) {
  auto mm = [](const std::vector<float>& a, float* lo, float* hi) {
    *lo = a[0];
    *hi = a[0];
    for (float v : a) {
      *lo = std::fmin(*lo, v);
      *hi = std::fmax(*hi, v);
    }
  };
  float xmin, xmax, ymin, ymax, zmin, zmax;
  mm(c.x, &xmin, &xmax);
  mm(c.y, &ymin, &ymax);
  mm(c.z, &zmin, &zmax);
  const int nk2 = g.nk + LENFD;
  for (int n = 0; n < s.num; ++n) {
    const float x0 = s.axis[3 * n], y0 = s.axis[3 * n + 1];
    float z0 = s.axis[3 * n + 2];
    if (x0 < xmin || x0 > xmax || y0 < ymin || y0 > ymax) continue;
    const int i = minloc_abs(c.x, x0), j = minloc_abs(c.y, y0);
    int k;
    if (z0 >= zmin && z0 <= zmax) {
      k = minloc_abs(c.z, z0);
    } else if (z0 > src_hyper_height) {
      k = nk2;
      z0 = c.z[k - 1];
    } else {
      continue;
    }
    if (i < LENFD + 1 || i > g.ni + LENFD || j < LENFD + 1 || j > g.nj + LENFD || k < LENFD + 1 || k > nk2) continue;
    s.found[n] = 1;
    s.indx[3 * n] = i;
    s.indx[3 * n + 1] = j;
    s.indx[3 * n + 2] = k;
    s.axis[3 * n + 2] = z0;
    s.shift[3 * n] = node_shift(c.x, i, x0);
    s.shift[3 * n + 1] = node_shift(c.y, j, y0);
    s.shift[3 * n + 2] = node_shift(c.z, k, z0);
  }
}

std::vector<double> as_double(const float* p, size_t n) { return std::vector<double>(p, p + n); }

// the variables of one source kind (all sources lie in the single rank's domain)
void put_sources(nc3::Writer& w, const char* kind, const char* const* comp, int ncomp, const Sources& s, int geo) {
  const std::string k = kind;
  const int dp = w.add_dim(k + "_point", s.num), dt = w.add_dim(k + "_time_window", s.ntw);
  for (int c = 0; c < ncomp; ++c) {
    std::vector<double> v(size_t(s.num) * s.ntw);
    for (int n = 0; n < s.num; ++n)
      for (int m = 0; m < s.ntw; ++m) v[size_t(n) * s.ntw + m] = s.val[(size_t(n) * ncomp + c) * s.ntw + m];
    w.add_var(comp[c], nc3::NC_FLOAT, {dp, dt}, v);
  }
  w.add_var(k + "_indx", nc3::NC_INT, {dp, geo}, std::vector<double>(s.indx.begin(), s.indx.end()));
  w.add_var(k + "_axis", nc3::NC_FLOAT, {dp, geo}, as_double(s.axis.data(), s.axis.size()));
  w.add_var(k + "_shift", nc3::NC_FLOAT, {dp, geo}, as_double(s.shift.data(), s.shift.size()));
  w.add_var(k + "_start_time", nc3::NC_FLOAT, {dp}, as_double(s.t0.data(), s.t0.size()));
  w.add_var(k + "_stf_time", nc3::NC_FLOAT, {dt}, as_double(s.time.data(), s.time.size()));
  w.add_var(k + "_stf_freq", nc3::NC_FLOAT, {dt}, as_double(s.freq.data(), s.freq.size()));
  w.add_gatt(k + "_stf_id", nc3::NC_INT, {double(s.stf_id)});
  for (const auto& e : STF_NAMES)
    if (e.id == s.stf_id) w.add_gatt_text(k + "_stf_type", e.name);
}

void stage_source(const conf::Text& cf) {
  const Grid g = main_grid(cf);
  conf::Text sc(cf.get("SOURCE_CONF", 2));
  const float src_hyper_height = getf(sc, "src_hyper_height", 2);
  Sources f, mo;
  f.num = sc.get_int("number_of_force_source", 2);
  if (f.num >= 1) read_forces(sc, f);
  else f.num = 0;
  mo.num = sc.get_int("number_of_moment_source", 2);
  if (mo.num >= 1) read_moments(sc, mo);
  else mo.num = 0;

  const Coord c = read_coord(cf, g);
  locate_sources(f, c, g, src_hyper_height);
  locate_sources(mo, c, g, src_hyper_height);
  bool missing = false;
  for (const Sources* s : {&f, &mo})
    for (int n = 0; n < s->num; ++n)
      if (!s->found[n]) {
        missing = true;
        std::printf(" n=%d loct= %.8g %.8g %.8g\n", n + 1, double(s->axis[3 * n]), double(s->axis[3 * n + 1]),
                    double(s->axis[3 * n + 2]));
      }
  if (missing) {
    std::printf(" there are some source points out of the computational domain\n");
    std::exit(1);
  }

  nc3::Writer w;
  const int geo = w.add_dim("geo_dimension", 3);
  w.add_gatt("number_of_force", nc3::NC_INT, {double(f.num)});
  w.add_gatt("number_of_moment", nc3::NC_INT, {double(mo.num)});
  static const char* const FCOMP[] = {"Fx", "Fy", "Fz"};
  static const char* const MCOMP[] = {"Mxx", "Myy", "Mzz", "Mxy", "Mxz", "Myz"};
  if (f.num > 0) put_sources(w, "force", FCOMP, 3, f, geo);
  if (mo.num > 0) put_sources(w, "moment", MCOMP, 6, mo, geo);
  write_or_die(w, cf.get("SOURCE_ROOT", 2) + "/source_" + SUFFIX + ".nc");
  std::printf("%d force and %d moment sources located\n", f.num, mo.num);
}

// ---- station: io_pt_read (mod_io.F90:112-152), receiver_locate (seis3d_station.F90:64-105)
// ---- and station_skel (:107-150) ----------------------------------------------------------

std::string io_enum(const char* prefix, int n) {
  char b[32];
  std::snprintf(b, sizeof b, "%s%03d", prefix, n);
  return b;
}

void stage_station(const conf::Text& cf) {
  const Grid g = main_grid(cf);
  const int num_recv = cf.get_int("number_of_recv", 2), num_line = cf.get_int("number_of_inline", 2);
  const int tinv = cf.get_int("tinv_of_seismo", 2);
  const float topo_hyper_height = getf(cf, "topo_hyper_height", 2);
  std::vector<float> xyz;  // (3, num_pt)
  std::vector<int> id;     // (2, num_pt)
  for (int n = 1; n <= num_recv; ++n) {
    for (int m = 0; m < 3; ++m) xyz.push_back(getf(cf, io_enum("recv_", n), m + 2));
    id.push_back(n);
    id.push_back(0);
  }
  for (int n = 1; n <= num_line; ++n) {
    const std::string key = io_enum("line_", n);
    float x0[3], dx[3];
    for (int m = 0; m < 3; ++m) {
      x0[m] = getf(cf, key, m + 2);
      dx[m] = getf(cf, key, m + 5);
    }
    const int npt = cf.get_int(key, 8);
    for (int m = 1; m <= npt; ++m) {
      for (int d = 0; d < 3; ++d) xyz.push_back(x0[d] + dx[d] * float(m - 1));
      id.push_back(m);
      id.push_back(n);
    }
  }
  const size_t num_pt = xyz.size() / 3;
  for (size_t n = 0; n < num_pt; ++n)
    for (int d = 0; d < 2; ++d) xyz[3 * n + d] = deg2rad_pt(xyz[3 * n + d]);

  const Coord c = read_coord(cf, g);
  const int nk2 = g.nk + LENFD;
  std::vector<double> indx, gindx, coord, grid, ids;
  for (size_t n = 0; n < num_pt; ++n) {
    const float x0 = xyz[3 * n], y0 = xyz[3 * n + 1], z0 = xyz[3 * n + 2];
    const int i = minloc_abs(c.x, x0), j = minloc_abs(c.y, y0);
    const int k = z0 <= topo_hyper_height ? minloc_abs(c.z, z0) : nk2;
    if (i < LENFD + 1 || i > g.ni + LENFD || j < LENFD + 1 || j > g.nj + LENFD || k < LENFD + 1 || k > nk2) continue;
    indx.insert(indx.end(), {double(i), double(j), double(k)});
    gindx.insert(gindx.end(), {double(i - LENFD), double(j - LENFD), double(k - LENFD)});  // out_i(swmpi_globi(i))
    coord.insert(coord.end(), {double(x0), double(y0), double(z0)});
    grid.insert(grid.end(), {double(c.x[i - 1]), double(c.y[j - 1]), double(c.z[k - 1])});
    ids.insert(ids.end(), {double(id[2 * n]), double(id[2 * n + 1])});
  }
  const size_t nrec = indx.size() / 3;
  nc3::Writer w;
  const int dn = w.add_dim("num_pt", 0), dg = w.add_dim("geo_dim", 3), d2 = w.add_dim("twoelem", 2);
  w.add_var("indx", nc3::NC_INT, {dn, dg}, indx);
  w.add_var("gindx", nc3::NC_INT, {dn, dg}, gindx);
  w.add_var("coord", nc3::NC_FLOAT, {dn, dg}, coord);
  w.add_var("grid", nc3::NC_FLOAT, {dn, dg}, grid);
  w.add_var("id", nc3::NC_INT, {dn, d2}, ids);
  w.add_gatt("tinv", nc3::NC_INT, {double(tinv)});
  w.set_numrecs(nrec);
  write_or_die(w, cf.get("STATION_ROOT", 2) + "/station_" + SUFFIX + ".nc");
  std::printf("%zu of %zu receivers located\n", nrec, num_pt);
}

int run(int argc, char** argv) {
  if (argc < 2) die("usage: fwant_prep grid|metric|source|station [SeisFD3D.conf] [--device N]");
  const std::string stage = argv[1];
  std::string conf_path = "SeisFD3D.conf";
  int device = 0;
  for (int a = 2; a < argc; ++a) {
    const std::string s = argv[a];
    if (s == "--device" && a + 1 < argc) device = std::atoi(argv[++a]);
    else conf_path = s;
  }
  const conf::Text cf(conf_path);
  if (stage == "grid") stage_grid(cf);
  else if (stage == "metric") stage_metric(cf, device);
  else if (stage == "source") stage_source(cf);
  else if (stage == "station") stage_station(cf);
  else die("unknown stage " + stage + " (grid, metric, source or station)");
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  try {
    return run(argc, argv);
  } catch (const std::exception& e) {
    die(e.what());
  }
}
