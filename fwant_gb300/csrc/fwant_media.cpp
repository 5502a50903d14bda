// fwant_media: the medium preprocessor stage as a program over the C ABI, a drop-in for
// the reference's seis3d_media (code/srcF/seis3d_media.F90) on one rank.
//
// Reads SeisFD3D.conf (ni, nj, nk, stept, dims, GRID_ROOT, MEDIA_CONF, MEDIA_ROOT:
// para_init / grid_fnm_init / media_fnm_init), the grid coordinates
// GRID_ROOT/coord_mpi000000.nc, the media configuration MEDIA_CONF (half_sample_point,
// background_type / _format / _filename, perturbed_type / _format / _filename:
// init_media :264-338) and the model file in its format: ascii cart1d, interface or layered
// files (layer1d_read :341-430, interface_read :433-532, layered_read :535-643) or NetCDF
// composite, volume or verpoly files (composite_read :646-702, volume_init / volume_read
// :705-779, verpoly_init / verpoly_read :782-850).  Evaluates the effective medium and the
// time-step limit on the GPU (fwant_media_*), writes MEDIA_ROOT/media_mpi000000.nc in the
// schema of media_create (:1346-1375: dimensions I, J, K with ghosts, the grid3d
// attributes, variables rho, lambda, mu) and prints the limit as the reference does
// (:235-244).
//
// Usage: fwant_media [SeisFD3D.conf] [--device N]
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "conf.h"
#include "fwant_media.h"
#include "netcdf3.h"

namespace {

constexpr double PI = 3.141592653589793;
const char* const SUFFIX = "mpi000000";

[[noreturn]] void die(const std::string& m) {
  std::fprintf(stderr, "fwant_media: %s\n", m.c_str());
  std::exit(1);
}

void check(fwant_status rc, fwant_media* m, const char* what) {
  if (rc != FWANT_OK) die(std::string(what) + ": " + (m ? fwant_media_last_error(m) : "failed"));
}

// ascii model files: string_conf keys and list-directed records after anchor lines
using TextModel = conf::Text;

// real(SP) array times a real(DP) factor, stored back in SP (L%Vp = L%Vp * v2ms)
void scale(std::vector<float>& a, double f) {
  for (float& v : a) v = float(double(v) * f);
}
// degrees to radians as the readers do (L%x = L%x * PI / 180.0_DP)
void to_rad(std::vector<float>& a) {
  for (float& v : a) v = float(double(v) * PI / 180.0);
}

void check_velocities(const std::vector<float>& vp, const std::vector<float>& vs, const std::vector<float>& dp,
                      const std::string& what, bool first_may_be_zero) {
  for (size_t q = 0; q < vp.size(); ++q) {
    if (first_may_be_zero && q == 0) {
      if (dp[q] < 0 || vp[q] < 0 || vs[q] < 0) die(what + ": model parameter should >=0 for (1,1)");
      continue;
    }
    if (dp[q] <= 0 || vp[q] <= 0 || vs[q] < 0) die(what + ": media parameter is negative");
    if (vp[q] * vp[q] <= 2.0f * (vs[q] * vs[q])) die(what + ": Vp**2 < 2Vs**2");
  }
}

struct Units {
  double d2m, v2ms, d2kgm3;
};
Units units(const TextModel& t) {
  return {t.get_double("distance2meter", 2), t.get_double("velocity2m/s", 2), t.get_double("density2kg/m^3", 2)};
}

// layer1d_read
void read_cart1d(fwant_media* m, const std::string& path) {
  TextModel t(path);
  const int kmax = t.get_int("radial_sampling", 2);
  if (kmax <= 1) die(path + ": sampling point should be larger than 1 for cart1d type");
  const Units u = units(t);
  std::vector<float> z(kmax), d(kmax), vp(kmax), vs(kmax), dp(kmax);
  t.seek("<anchor_data>");
  for (int k = 0; k < kmax; ++k) {
    const auto r = t.record(4);
    z[k] = r[0];
    dp[k] = r[1];
    vp[k] = r[2];
    vs[k] = r[3];
  }
  scale(vp, u.v2ms);
  scale(vs, u.v2ms);
  scale(dp, u.d2kgm3);
  check_velocities(vp, vs, dp, path, false);
  const std::string meaning = t.get("radial_meaning", 2);
  if (meaning == "axis") {
    const double d0 = std::max(z[0], z[kmax - 1]);
    for (int k = 0; k < kmax; ++k) d[k] = float(d0 - double(z[k]));
  } else if (meaning == "thickness") {
    d[0] = 0.0f;
    for (int k = 1; k < kmax; ++k) d[k] = z[k - 1] + d[k - 1];
  } else if (meaning == "depth") {
    d = z;  // the reference leaves d unset for 'depth'; the values are depths
  } else {
    die(path + ": layer_meaning can only take axis, depth or thickness");
  }
  if (d[0] > d[kmax - 1])
    for (auto* a : {&d, &vp, &vs, &dp}) std::reverse(a->begin(), a->end());
  scale(d, u.d2m);
  check(fwant_media_set_cart1d(m, kmax, d.data(), vp.data(), vs.data(), dp.data()), m, "cart1d");
}

// the (2, kmax) value pairs after <anchor_media>: each record Vp(1:2) Vs(1:2) Dp(1:2)
void read_pairs(TextModel& t, int kmax, const Units& u, std::vector<float>& vp, std::vector<float>& vs,
                std::vector<float>& dp) {
  vp.assign(size_t(2) * kmax, 0.0f);
  vs = vp;
  dp = vp;
  t.seek("<anchor_media>");
  for (int k = 0; k < kmax; ++k) {
    const auto r = t.record(6);
    for (int s = 0; s < 2; ++s) {
      vp[2 * k + s] = r[s];
      vs[2 * k + s] = r[2 + s];
      dp[2 * k + s] = r[4 + s];
    }
  }
  scale(vp, u.v2ms);
  scale(vs, u.v2ms);
  scale(dp, u.d2kgm3);
}

// interface_read and layered_read; `interface`: z of each interface, else h or d per layer
void read_layers(fwant_media* m, const std::string& path, bool interface) {
  TextModel t(path);
  const int kmax = t.get_int(interface ? "number_of_interface" : "number_of_layer", 2);
  if (kmax < 1) die(path + ": at least 1 layer should exist");
  const Units u = units(t);
  const int imax = t.get_int("horizontal_sampling", 2), jmax = t.get_int("horizontal_sampling", 3);
  if (imax < 2 || jmax < 2) die(path + ": horizontal_sampling must be at least 2 x 2");
  std::vector<float> vp, vs, dp;
  read_pairs(t, kmax, u, vp, vs, dp);
  if (interface) {
    check_velocities(vp, vs, dp, path, true);
  } else {
    check_velocities(vp, vs, dp, path, false);
  }
  const size_t plane = size_t(imax) * jmax, n3 = plane * kmax;
  std::vector<float> x(imax), y(jmax), z(n3, 0.0f), h(n3, 0.0f);
  std::string meaning = "depth";
  if (!interface) {
    meaning = t.get("layer_meaning", 2);
    if (meaning != "depth" && meaning != "thickness") die(path + ": layer_meaning can only take depth or thickness");
  }
  t.seek(interface ? "<anchor_interface>" : "<anchor_layer>");
  for (int j = 0; j < jmax; ++j)
    for (int i = 0; i < imax; ++i) {
      const auto r = t.record(size_t(2) + kmax);
      x[i] = r[0];
      y[j] = r[1];
      for (int k = 0; k < kmax; ++k) (interface || meaning == "depth" ? z : h)[plane * k + size_t(j) * imax + i] = r[2 + k];
    }
  if (interface) {
    for (int k = 0; k + 1 < kmax; ++k)
      for (size_t p = 0; p < plane; ++p) h[plane * k + p] = z[plane * k + p] - z[plane * (k + 1) + p];
    for (size_t p = 0; p + plane < n3; ++p)
      if (h[p] < 0.0f) die(path + ": thickness btween two interfaces shouldn' be less than 0");
  } else if (meaning == "depth") {  // z holds the depths d
    for (size_t p = 0; p < plane; ++p) h[p] = z[p];
    for (int k = 1; k < kmax; ++k)
      for (size_t p = 0; p < plane; ++p) h[plane * k + p] = z[plane * k + p] - z[plane * (k - 1) + p];
  }
  if (!interface) {
    for (size_t p = 0; p + plane < n3; ++p)
      if (h[p] < 0.0f) die(path + ": thickness of layer should not be less than 0");
    for (size_t p = n3 - plane; p < n3; ++p)
      if (h[p] < 1.0e-20f) die(path + ": thickness of lowest layer should larger than 0");
  }
  to_rad(x);
  to_rad(y);
  scale(z, u.d2m);
  scale(h, u.d2m);
  check(fwant_media_set_layers(m, interface ? FWANT_MEDIA_INTERFACE : FWANT_MEDIA_LAYERED, imax, jmax, kmax, x.data(),
                               y.data(), interface ? z.data() : nullptr, h.data(), vp.data(), vs.data(), dp.data(),
                               nullptr, nullptr, nullptr),
        m, interface ? "interface" : "layered");
}

std::vector<float> nc_var(const nc3::Reader& f, const std::string& path, const std::string& name, size_t n) {
  std::vector<float> v;
  std::string err;
  if (!f.read(name, &v, &err)) die(path + ": " + err);
  if (v.size() != n) die(path + ": variable " + name + " has " + std::to_string(v.size()) + " values, expected " +
                         std::to_string(n));
  return v;
}

int nc_dim(const nc3::Reader& f, const std::string& path, const std::string& name) {
  const nc3::Dim* d = f.dim(name);
  if (!d) die(path + ": no dimension " + name);
  return int(d->len);
}

float nc_gatt(const nc3::Reader& f, const std::string& path, const std::string& name) {
  const nc3::Att* a = f.gatt(name);
  if (!a || a->num.empty()) die(path + ": no attribute " + name);
  return float(a->num[0]);
}

void open_nc(nc3::Reader& f, const std::string& path) {
  std::string err;
  if (!f.open(path, &err)) die(err);
}

// composite_read
void read_composite(fwant_media* m, const std::string& path) {
  nc3::Reader f;
  open_nc(f, path);
  const int imax = nc_dim(f, path, "theta"), jmax = nc_dim(f, path, "phi"), kmax = nc_dim(f, path, "layer");
  const size_t n3 = size_t(imax) * jmax * kmax;
  auto x = nc_var(f, path, "theta", imax), y = nc_var(f, path, "phi", jmax);
  const auto h = nc_var(f, path, "thickness", n3);
  const auto vp = nc_var(f, path, "Vp", 2 * n3), vs = nc_var(f, path, "Vs", 2 * n3), dp = nc_var(f, path, "rho", 2 * n3);
  const auto ep = nc_var(f, path, "Vp_poly_d", kmax), es = nc_var(f, path, "Vs_poly_d", kmax),
             er = nc_var(f, path, "rho_poly_d", kmax);
  to_rad(x);
  to_rad(y);
  const size_t plane = size_t(imax) * jmax;
  for (size_t p = 0; p + plane < n3; ++p)
    if (h[p] < 0.0f) die(path + ": thickness of layer should not be less than 0");
  for (size_t p = n3 - plane; p < n3; ++p)
    if (h[p] < 1.0e-20f) die(path + ": thickness of lowest layer should larger than 0");
  check(fwant_media_set_layers(m, FWANT_MEDIA_COMPOSITE, imax, jmax, kmax, x.data(), y.data(), nullptr, h.data(),
                               vp.data(), vs.data(), dp.data(), ep.data(), es.data(), er.data()),
        m, "composite");
}

// volume_init + volume_read (the sub-volume is selected inside the library)
void read_volume(fwant_media* m, const std::string& path, int perturbed) {
  nc3::Reader f;
  open_nc(f, path);
  const int imax = nc_dim(f, path, "theta"), jmax = nc_dim(f, path, "phi"), kmax = nc_dim(f, path, "depth");
  const size_t n3 = size_t(imax) * jmax * kmax;
  auto x = nc_var(f, path, "theta", imax), y = nc_var(f, path, "phi", jmax);
  const auto rz = nc_var(f, path, "depth2sealevel", kmax);
  const float rz0 = nc_gatt(f, path, "sealevel");
  const auto vp = nc_var(f, path, "Vp", n3), vs = nc_var(f, path, "Vs", n3), dp = nc_var(f, path, "rho", n3);
  to_rad(x);
  to_rad(y);
  check(fwant_media_set_volume(m, perturbed, imax, jmax, kmax, x.data(), y.data(), rz.data(), rz0, vp.data(),
                               vs.data(), dp.data()),
        m, "volume");
}

// verpoly_init + verpoly_read
void read_verpoly(fwant_media* m, const std::string& path, int perturbed) {
  nc3::Reader f;
  open_nc(f, path);
  const int imax = nc_dim(f, path, "theta"), jmax = nc_dim(f, path, "phi"), kmax = nc_dim(f, path, "depth"),
            nmax = nc_dim(f, path, "polynomial");
  const size_t n3 = size_t(imax) * jmax * kmax;
  auto x = nc_var(f, path, "theta", imax), y = nc_var(f, path, "phi", jmax);
  const auto ep = nc_var(f, path, "Vp_poly_d", nmax), es = nc_var(f, path, "Vs_poly_d", nmax),
             er = nc_var(f, path, "rho_poly_d", nmax);
  const float rz0 = nc_gatt(f, path, "sealevel");
  const auto rz = nc_var(f, path, "depth2sealevel", n3);
  const auto cp = nc_var(f, path, "Vp_poly_c", n3 * nmax), cs = nc_var(f, path, "Vs_poly_c", n3 * nmax),
             cr = nc_var(f, path, "rho_poly_c", n3 * nmax);
  to_rad(x);
  to_rad(y);
  check(fwant_media_set_verpoly(m, perturbed, imax, jmax, kmax, nmax, x.data(), y.data(), rz.data(), rz0, cp.data(),
                                cs.data(), cr.data(), ep.data(), es.data(), er.data()),
        m, "verpoly");
}

void read_model(fwant_media* m, const std::string& type, const std::string& format, const std::string& file,
                int perturbed) {
  const bool ascii = type == "cart1d" || type == "interface" || type == "layered";
  if (ascii && format != "ascii") die("only ascii input accepted for " + type + " type");
  if (!ascii && format != "nc") die("only nc input accepted for " + type + " type");
  if (perturbed && type != "volume" && type != "verpoly") die("perturbed_type must be volume, verpoly or none");
  if (type == "cart1d") read_cart1d(m, file);
  else if (type == "interface") read_layers(m, file, true);
  else if (type == "layered") read_layers(m, file, false);
  else if (type == "composite") read_composite(m, file);
  else if (type == "volume") read_volume(m, file, perturbed);
  else if (type == "verpoly") read_verpoly(m, file, perturbed);
  else die("unknown model type " + type);
}

}  // namespace

static int run(int argc, char** argv) {
  std::string conf_path = "SeisFD3D.conf";
  int device = 0;
  for (int a = 1; a < argc; ++a) {
    const std::string s = argv[a];
    if (s == "--device" && a + 1 < argc) device = std::atoi(argv[++a]);
    else conf_path = s;
  }
  conf::File cf;
  std::string err;
  if (!cf.load(conf_path, &err)) die(err);
  auto need_i = [&](const std::string& k, int col) {
    int v;
    if (!cf.get_int(k, col, &v)) die(conf_path + ": key " + k + " missing");
    return v;
  };
  auto need_s = [&](conf::File& f, const std::string& path, const std::string& k, int col) {
    std::string v;
    if (!f.get(k, col, &v)) die(path + ": key " + k + " missing");
    return v;
  };
  const int ni = need_i("ni", 2), nj = need_i("nj", 2), nk = need_i("nk", 2);
  double stept = 0.0;
  if (!cf.get_double("stept", 2, &stept)) die(conf_path + ": key stept missing");
  if (cf.has("dims"))
    for (int d = 0; d < 3; ++d)
      if (need_i("dims", d + 2) != 1) die("dims must be 1 1 1: one GPU evaluates the whole grid");
  const std::string grid_root = need_s(cf, conf_path, "GRID_ROOT", 2), media_conf = need_s(cf, conf_path, "MEDIA_CONF", 2),
                    media_root = need_s(cf, conf_path, "MEDIA_ROOT", 2);
  const int nx = ni + 6, ny = nj + 6, nz = nk + 6;

  // grid_coord_import
  nc3::Reader fc;
  const std::string pc = grid_root + "/coord_" + SUFFIX + ".nc";
  open_nc(fc, pc);
  const auto x = nc_var(fc, pc, "x", nx), y = nc_var(fc, pc, "y", ny), z = nc_var(fc, pc, "z", nz);
  const float ztopo = z[3 + nk - 1];

  // init_media
  conf::File mc;
  if (!mc.load(media_conf, &err)) die(err);
  int half[3];
  for (int d = 0; d < 3; ++d)
    if (!mc.get_int("half_sample_point", d + 2, &half[d])) die(media_conf + ": key half_sample_point missing");
  fwant_media* m = nullptr;
  check(fwant_media_create(ni, nj, nk, x.data(), y.data(), z.data(), ztopo, half, device, &m), nullptr, "create");
  std::printf("init media ...\n");
  read_model(m, need_s(mc, media_conf, "background_type", 2), need_s(mc, media_conf, "background_format", 2),
             need_s(mc, media_conf, "background_filename", 2), 0);
  const std::string ptype = need_s(mc, media_conf, "perturbed_type", 2);
  if (ptype != "none")
    read_model(m, ptype, need_s(mc, media_conf, "perturbed_format", 2), need_s(mc, media_conf, "perturbed_filename", 2),
               1);

  // effmedia_eval + media_extend
  std::printf("calculate effective media ...\n");
  const size_t n3 = size_t(nx) * ny * nz;
  std::vector<float> lam(n3), mu(n3), rho(n3);
  check(fwant_media_eval(m, lam.data(), mu.data(), rho.data()), m, "effective media");

  // media_create: nfseis_grid3d_skel + nfseis_grid3d_attput + rho, lambda, mu
  std::printf("  export media...\n");
  {
    nc3::Writer w;
    const int dI = w.add_dim("I", nx), dJ = w.add_dim("J", ny), dK = w.add_dim("K", nz);
    w.add_gatt_text("title", "media generated by seis3d_media");
    const int ni1 = 4, ni2 = ni + 3, nj1 = 4, nj2 = nj + 3, nk1 = 4, nk2 = nk + 3;
    const std::pair<const char*, int> atts[] = {
        {"ni1", ni1}, {"ni2", ni2}, {"nj1", nj1}, {"nj2", nj2}, {"nk1", nk1}, {"nk2", nk2}, {"ni", ni},
        {"nj", nj},   {"nk", nk},   {"nx1", 1},   {"nx2", nx},  {"ny1", 1},   {"ny2", ny},  {"nz1", 1},
        {"nz2", nz},  {"nx", nx},   {"ny", ny},   {"nz", nz},   {"ngi1", ni1}, {"ngi2", ni2}, {"ngj1", nj1},
        {"ngj2", nj2}, {"ngk1", nk1}, {"ngk2", nk2}, {"ngx1", 1}, {"ngx2", nx}, {"ngy1", 1}, {"ngy2", ny},
        {"ngz1", 1},  {"ngz2", nz}};
    for (const auto& a : atts) w.add_gatt(a.first, nc3::NC_INT, {double(a.second)});
    w.add_gatt("point_in_this", nc3::NC_INT, {double(ni1), double(ni2), double(nj1), double(nj2), double(nk1), double(nk2)});
    w.add_gatt("start", nc3::NC_INT, {1, 1, 1});
    w.add_gatt("count", nc3::NC_INT, {double(nx), double(ny), double(nz)});
    w.add_gatt("stride", nc3::NC_INT, {1, 1, 1});
    w.add_var_f("rho", {dK, dJ, dI}, rho.data(), n3);
    w.add_var_f("lambda", {dK, dJ, dI}, lam.data(), n3);
    w.add_var_f("mu", {dK, dJ, dI}, mu.data(), n3);
    const std::string out = media_root + "/media_" + SUFFIX + ".nc";
    if (!w.write(out, &err)) die(err);
  }

  // media_stept_check and the report of the main program
  float dtmax = 0.0f, vp = 0.0f, dl = 0.0f;
  int ijk[3] = {0, 0, 0};
  check(fwant_media_stept_check(m, &dtmax, ijk, &vp, &dl), m, "time-step check");
  double ms = 0.0;
  fwant_media_last_eval_ms(m, &ms);
  std::printf("Maximum allowed time step is %.8g\n", double(dtmax));
  std::printf("located on%5d%5d%5d in thread%5d%5d%5d\n", ijk[0], ijk[1], ijk[2], 0, 0, 0);
  std::printf(" Vp and dL are: %.8g %.8g\n", double(vp), double(dl));
  if (double(dtmax) < stept) std::printf("Serious Error: stept>dtmax %.8g %.8g\n", stept, double(dtmax));
  std::printf("effective media on the GPU: %.3f ms\n", ms);
  fwant_media_destroy(m);
  return 0;
}

int main(int argc, char** argv) {
  try {
    return run(argc, argv);
  } catch (const std::exception& e) {
    die(e.what());
  }
}
