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
//   fwant_prep stitch  [SeisFD3D.conf] --out DIR     the per-rank files of a dims > 1 input set
//                                                    -> DIR/{coord,metric,media,source,station}_mpi000000.nc
//                                                       and DIR/SeisFD3D.conf (one rank)
//
// grid, source and station run on the host (a few thousand coordinates and a handful of
// points); metric evaluates the FP64 metric on the GPU (fwant_metric_arrays).  Every FP32
// expression is evaluated in the reference's order and precision (this file is compiled
// without contraction), so the files hold the values the reference's programs write.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
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


// ---- stitch: a multi-rank input set (dims > 1) as the one-rank set of the same grid -------
//
// The reference's preprocessors write one file per rank (set_mpi_subfix, mod_mpi.F90:415-423:
// coord_mpiIIJJKK.nc ...), each over the rank's local arrays with ghosts: rank (a, b, c) of
// dims (da, db, dc) holds global points a*ni + l, l = 0 .. ni+5 (0-based, ghosts included;
// swmpi_globi, mod_mpi.F90:450-454), with ni the per-rank size of SeisFD3D.conf.  The
// stitched grid has NI = ni*da points and takes every point from the rank that owns it as
// an interior point (the outer ghost planes from the edge ranks): a rank's own ghost values
// can differ from its neighbour's interior ones (seis3d_metric's one-sided stencils at the
// local ends).  Sources are listed by every rank whose points with ghosts hold their centre
// (seis3d_source.F90:186-293) with local indices: they are mapped to global indices and
// kept once, in rank order.  Receivers are listed by the one rank whose interior holds them
// (seis3d_station.F90:64-105): mapped and concatenated in rank order.
std::string rank_suffix(int a, int b, int c) {
  char buf[40];  // dims are at most 99 per direction: two digits each (i2.2)
  std::snprintf(buf, sizeof buf, "mpi%02d%02d%02d", a, b, c);
  return buf;
}

struct RankFile {
  int r[3];
  nc3::Reader f;
  std::string path;
};

void stage_stitch(const std::string& conf_path, const std::string& out_dir) {
  const conf::Text cf(conf_path);
  const int n[3] = {cf.get_int("ni", 2), cf.get_int("nj", 2), cf.get_int("nk", 2)};
  int dims[3] = {1, 1, 1};
  if (cf.has("dims"))
    for (int d = 0; d < 3; ++d) dims[d] = cf.get_int("dims", d + 2);
  for (int d = 0; d < 3; ++d)
    if (n[d] < 2 || dims[d] < 1 || dims[d] > 99) die(conf_path + ": ni, nj, nk >= 2 and dims 1 .. 99");
  const int N[3] = {n[0] * dims[0], n[1] * dims[1], n[2] * dims[2]};
  const int X[3] = {N[0] + 2 * LENFD, N[1] + 2 * LENFD, N[2] + 2 * LENFD};       // stitched with ghosts
  const int lx[3] = {n[0] + 2 * LENFD, n[1] + 2 * LENFD, n[2] + 2 * LENFD};      // one rank with ghosts
  // owner rank and local index of global index G (0-based with ghosts) along axis d
  auto owner = [&](int d, int G, int* l) {
    int r = (G - LENFD) / n[d];
    if (G < LENFD) r = 0;
    if (r > dims[d] - 1) r = dims[d] - 1;
    *l = G - r * n[d];
    return r;
  };
  auto open_all = [&](const std::string& root, const std::string& prefix) {
    std::vector<RankFile> files;
    files.reserve(size_t(dims[0]) * dims[1] * dims[2]);  // the readers own open files: never relocated
    for (int a = 0; a < dims[0]; ++a)
      for (int b = 0; b < dims[1]; ++b)
        for (int c = 0; c < dims[2]; ++c) {
          files.emplace_back();
          RankFile& rf = files.back();
          rf.r[0] = a; rf.r[1] = b; rf.r[2] = c;
          rf.path = root + "/" + prefix + "_" + rank_suffix(a, b, c) + ".nc";
          std::string err;
          if (!rf.f.open(rf.path, &err)) die(err);
        }
    return files;
  };
  auto rank_of = [&](const std::vector<RankFile>& files, int a, int b, int c) -> const RankFile& {
    return files[size_t((a * dims[1] + b) * dims[2] + c)];
  };
  auto read_d = [&](const RankFile& rf, const std::string& name) {
    std::vector<double> v;
    std::string err;
    if (!rf.f.read(name, &v, &err)) die(rf.path + ": " + err);
    return v;
  };
  const std::string grid_atts[] = {"ni1", "ni2", "nj1", "nj2", "nk1", "nk2", "ni", "nj", "nk", "nx1", "nx2",
                                   "ny1", "ny2", "nz1", "nz2", "nx", "ny", "nz", "ngi1", "ngi2", "ngj1", "ngj2",
                                   "ngk1", "ngk2", "ngx1", "ngx2", "ngy1", "ngy2", "ngz1", "ngz2"};
  auto grid_att_value = [&](const std::string& name) -> double {
    const int ax = name.find('i') != std::string::npos || name.find('x') != std::string::npos ? 0
                   : (name.find('j') != std::string::npos || name.find('y') != std::string::npos ? 1 : 2);
    const bool ghosts = name.find('x') != std::string::npos || name.find('y') != std::string::npos ||
                        name.find('z') != std::string::npos;
    const char last = name.back();
    if (last == '1') return ghosts ? 1 : LENFD + 1;
    if (last == '2') return ghosts ? X[ax] : LENFD + N[ax];
    return ghosts ? X[ax] : N[ax];
  };
  // grid-shaped files: every variable over I, J and/or K is assembled point by point
  auto stitch_grid = [&](const std::string& root, const std::string& prefix) {
    std::vector<RankFile> files = open_all(root, prefix);
    const nc3::Reader& f0 = files[0].f;
    nc3::Writer w;
    std::vector<int> dim_axis;  // per dimension of rank 0's file: axis 0..2 or -1
    for (const nc3::Dim& dm : f0.dims) {
      const int ax = dm.name == "I" ? 0 : (dm.name == "J" ? 1 : (dm.name == "K" ? 2 : -1));
      if (ax >= 0 && dm.len != uint64_t(lx[ax])) die(files[0].path + ": dimension " + dm.name + " is not n + 6");
      dim_axis.push_back(ax);
      w.add_dim(dm.name, ax >= 0 ? uint64_t(X[ax]) : dm.len);
    }
    for (const nc3::Att& at : f0.gatts) {
      bool grid = false;
      for (const std::string& g : grid_atts) grid = grid || at.name == g;
      if (at.type == nc3::NC_CHAR) w.add_gatt_text(at.name, at.text);
      else if (grid) w.add_gatt(at.name, at.type, {grid_att_value(at.name)});
      else if (at.name == "point_in_this")
        w.add_gatt(at.name, at.type, {double(LENFD + 1), double(LENFD + N[0]), double(LENFD + 1), double(LENFD + N[1]),
                                      double(LENFD + 1), double(LENFD + N[2])});
      else if (at.name == "count") w.add_gatt(at.name, at.type, {double(X[0]), double(X[1]), double(X[2])});
      else w.add_gatt(at.name, at.type, at.num);
    }
    for (const nc3::Var& v : f0.vars) {
      // the variable's axes, slowest first; a dimension that is not I, J, K must have length 1
      std::vector<int> axes;
      for (int d : v.dims) {
        if (dim_axis[size_t(d)] < 0 && f0.dims[size_t(d)].len != 1)
          die(files[0].path + ": variable " + v.name + " has a non-grid dimension");
        axes.push_back(dim_axis[size_t(d)]);
      }
      std::vector<std::vector<double>> local(files.size());
      for (size_t q = 0; q < files.size(); ++q) local[q] = read_d(files[q], v.name);
      size_t total = 1;
      for (int ax : axes) total *= ax >= 0 ? size_t(X[ax]) : 1;
      std::vector<double> out(total);
      std::vector<int> G(axes.size(), 0);
      for (size_t e = 0; e < total; ++e) {
        // decompose e (last dimension fastest) into global indices
        size_t rem = e;
        for (size_t q = axes.size(); q-- > 0;) {
          const int len = axes[q] >= 0 ? X[axes[q]] : 1;
          G[q] = int(rem % size_t(len));
          rem /= size_t(len);
        }
        int r[3] = {0, 0, 0}, l[3] = {0, 0, 0};
        for (size_t q = 0; q < axes.size(); ++q)
          if (axes[q] >= 0) r[axes[q]] = owner(axes[q], G[q], &l[axes[q]]);
        const RankFile& rf = rank_of(files, r[0], r[1], r[2]);
        size_t le = 0;
        for (size_t q = 0; q < axes.size(); ++q) le = le * size_t(axes[q] >= 0 ? lx[axes[q]] : 1) + size_t(axes[q] >= 0 ? l[axes[q]] : 0);
        out[e] = local[size_t(&rf - files.data())][le];
      }
      std::vector<int> vdims(v.dims.begin(), v.dims.end());
      w.add_var(v.name, v.type, vdims, out);
    }
    write_or_die(w, out_dir + "/" + prefix + "_" + SUFFIX + ".nc");
  };
  stitch_grid(cf.get("GRID_ROOT", 2), "coord");
  stitch_grid(cf.get("GRID_ROOT", 2), "metric");
  stitch_grid(cf.get("MEDIA_ROOT", 2), "media");

  // list-shaped files: the records of every rank, indices mapped to the stitched grid
  auto map_indx = [&](std::vector<double>& v, const RankFile& rf) {
    for (size_t e = 0; e < v.size(); ++e) v[e] += double(rf.r[e % 3] * n[e % 3]);
  };
  // sources: per kind (force, moment), the records in rank order, each kept once
  {
    std::vector<RankFile> files = open_all(cf.get("SOURCE_ROOT", 2), "source");
    const nc3::Reader& f0 = files[0].f;
    nc3::Writer w;
    std::vector<int> dmap(f0.dims.size());
    struct Kind {
      std::string k;
      std::vector<std::vector<double>> recs;  // per kept source: all its values, variable after variable
      int ntw = 0;
    };
    Kind kinds[2] = {{"force"}, {"moment"}};
    for (Kind& kd : kinds) {
      const nc3::Dim* tw = f0.dim(kd.k + "_time_window");
      if (!tw) continue;
      kd.ntw = int(tw->len);
    }
    // per kind the point-dimensioned variables in rank 0's order
    auto point_vars = [&](const std::string& k) {
      std::vector<const nc3::Var*> vs;
      const nc3::Dim* pd = f0.dim(k + "_point");
      if (!pd) return vs;
      const int pid = int(pd - f0.dims.data());
      for (const nc3::Var& v : f0.vars)
        if (!v.dims.empty() && v.dims[0] == pid) vs.push_back(&v);
      return vs;
    };
    for (Kind& kd : kinds) {
      if (!f0.dim(kd.k + "_point")) continue;
      const std::vector<const nc3::Var*> vs = point_vars(kd.k);
      for (const RankFile& rf : files) {
        const nc3::Dim* pd = rf.f.dim(kd.k + "_point");
        const size_t np = pd ? size_t(pd->len) : 0;
        if (np == 0) continue;
        std::vector<std::vector<double>> vals;
        for (const nc3::Var* v : vs) {
          std::vector<double> a = read_d(rf, v->name);
          if (v->name == kd.k + "_indx") map_indx(a, rf);
          vals.push_back(std::move(a));
        }
        for (size_t p = 0; p < np; ++p) {
          std::vector<double> rec;
          for (const std::vector<double>& a : vals) {
            const size_t per = a.size() / np;
            rec.insert(rec.end(), a.begin() + ptrdiff_t(p * per), a.begin() + ptrdiff_t((p + 1) * per));
          }
          bool seen = false;
          for (const auto& r : kd.recs) seen = seen || r == rec;
          if (!seen) kd.recs.push_back(std::move(rec));
        }
      }
    }
    for (size_t d = 0; d < f0.dims.size(); ++d) {
      const nc3::Dim& dm = f0.dims[d];
      uint64_t len = dm.len;
      for (const Kind& kd : kinds)
        if (dm.name == kd.k + "_point") len = kd.recs.size();
      dmap[d] = w.add_dim(dm.name, len);
    }
    for (const nc3::Att& at : f0.gatts) {
      if (at.type == nc3::NC_CHAR) w.add_gatt_text(at.name, at.text);
      else if (at.name == "number_of_force") w.add_gatt(at.name, at.type, {double(kinds[0].recs.size())});
      else if (at.name == "number_of_moment") w.add_gatt(at.name, at.type, {double(kinds[1].recs.size())});
      else w.add_gatt(at.name, at.type, at.num);
    }
    for (const nc3::Var& v : f0.vars) {
      std::vector<int> vdims;
      for (int d : v.dims) vdims.push_back(dmap[size_t(d)]);
      const Kind* kd = nullptr;
      size_t off = 0, per = 0;
      for (const Kind& k : kinds) {
        const std::vector<const nc3::Var*> vs = point_vars(k.k);
        size_t o = 0;
        for (const nc3::Var* pv : vs) {
          size_t each = 1;
          for (size_t q = 1; q < pv->dims.size(); ++q) each *= size_t(f0.dims[size_t(pv->dims[q])].len);
          if (pv == &v) { kd = &k; off = o; per = each; }
          o += each;
        }
      }
      std::vector<double> out;
      if (kd) {
        for (const auto& rec : kd->recs) out.insert(out.end(), rec.begin() + ptrdiff_t(off), rec.begin() + ptrdiff_t(off + per));
      } else {
        out = read_d(files[0], v.name);  // per-window tables, the same in every rank's file
      }
      w.add_var(v.name, v.type, vdims, out);
    }
    write_or_die(w, out_dir + "/source_" + SUFFIX + ".nc");
  }
  // receivers: every rank's records in rank order
  {
    std::vector<RankFile> files = open_all(cf.get("STATION_ROOT", 2), "station");
    const nc3::Reader& f0 = files[0].f;
    nc3::Writer w;
    std::vector<std::vector<double>> cols(f0.vars.size());
    size_t total = 0;
    for (const RankFile& rf : files) {
      const size_t np = size_t(rf.f.numrecs());
      total += np;
      for (size_t q = 0; q < f0.vars.size(); ++q) {
        if (np == 0) continue;
        std::vector<double> a = read_d(rf, f0.vars[q].name);
        if (f0.vars[q].name == "indx") map_indx(a, rf);
        cols[q].insert(cols[q].end(), a.begin(), a.end());
      }
    }
    std::vector<int> dmap;
    for (const nc3::Dim& dm : f0.dims) dmap.push_back(w.add_dim(dm.name, dm.len));
    for (const nc3::Att& at : f0.gatts) {
      if (at.type == nc3::NC_CHAR) w.add_gatt_text(at.name, at.text);
      else w.add_gatt(at.name, at.type, at.num);
    }
    for (size_t q = 0; q < f0.vars.size(); ++q) {
      std::vector<int> vdims;
      for (int d : f0.vars[q].dims) vdims.push_back(dmap[size_t(d)]);
      w.add_var(f0.vars[q].name, f0.vars[q].type, vdims, cols[q]);
    }
    w.set_numrecs(total);
    write_or_die(w, out_dir + "/station_" + SUFFIX + ".nc");
  }
  // the one-rank configuration: the same file with the stitched sizes, dims 1 1 1 and the
  // input roots pointing at out_dir
  {
    std::ifstream in(conf_path);
    std::ofstream out(out_dir + "/SeisFD3D.conf");
    if (!in || !out) die("cannot copy " + conf_path + " to " + out_dir);
    const std::string nv[3] = {std::to_string(N[0]), std::to_string(N[1]), std::to_string(N[2])};
    for (std::string line; std::getline(in, line);) {
      const size_t eq = line.find('=');
      std::string key = eq == std::string::npos ? "" : line.substr(0, eq);
      key.erase(0, key.find_first_not_of(" \t"));
      key.erase(key.find_last_not_of(" \t") + 1);
      if (key == "ni" || key == "nj" || key == "nk")
        line = key + " = " + nv[key == "ni" ? 0 : (key == "nj" ? 1 : 2)];
      else if (key == "dims")
        line = "dims = 1 1 1";
      else if (key == "GRID_ROOT" || key == "MEDIA_ROOT" || key == "SOURCE_ROOT" || key == "STATION_ROOT")
        line = key + " = " + out_dir;
      out << line << "\n";
    }
  }
  std::printf("stitched %d x %d x %d ranks into one %d x %d x %d grid in %s\n", dims[0], dims[1], dims[2], N[0], N[1],
              N[2], out_dir.c_str());
}

int run(int argc, char** argv) {
  if (argc < 2) die("usage: fwant_prep grid|metric|source|station|stitch [SeisFD3D.conf] [--device N] [--out DIR]");
  const std::string stage = argv[1];
  std::string conf_path = "SeisFD3D.conf", out_dir;
  int device = 0;
  for (int a = 2; a < argc; ++a) {
    const std::string s = argv[a];
    if (s == "--device" && a + 1 < argc) device = std::atoi(argv[++a]);
    else if (s == "--out" && a + 1 < argc) out_dir = argv[++a];
    else conf_path = s;
  }
  if (stage == "stitch") {
    if (out_dir.empty()) die("stitch: --out DIR is required");
    stage_stitch(conf_path, out_dir);
    return 0;
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
