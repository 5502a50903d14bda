// fwant_wave — the solver stage as a program: reads the same SeisFD3D.conf keys and the
// same per-rank NetCDF input files as the reference's seis3d_wave_mpi
// (code/srcF/seis3d_wave_8op_p3.F90:50-80: para_init, io_init, grid/metric/media/source/
// station imports, abs_init, io_snap_read), runs the time loop on one GPU through the
// C ABI, and writes the same output files: seismo_mpi000000.nc (io_seismo_*,
// code/srcF/mod_io.F90:429-497) and the vel_/sgt_ snapshot files (io_wave_export,
// code/srcF/mod_io.F90:505-645).  One rank: `dims` must be 1 1 1 and every file name
// carries the suffix mpi000000.
//
// Checkpoints (CHECKPOINT_ROOT, checkpoint_tinv, run_from_checkpoint) use the library's
// complete-state format (rest_tNNNNN_mpi000000.ckpt) instead of the reference's
// fields-only NetCDF restart files, so a resumed run repeats the uninterrupted one exactly.
//
// Also: --nc-copy IN OUT re-writes a NetCDF file through this program's reader and
// writer; --nc-dump FILE prints its header and per-variable sums (format checks).
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <map>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/fwant_gb300.h"
#include "conf.h"
#include "netcdf3.h"
#include "seisfd_conf.h"

namespace {

const char* const SUFFIX = seisfd::MPI_SUFFIX;
const char* const COMP[9] = {"Vx", "Vy", "Vz", "Txx", "Tyy", "Tzz", "Txy", "Txz", "Tyz"};

[[noreturn]] void die(const std::string& msg) {
  std::fprintf(stderr, "fwant_wave: %s\n", msg.c_str());
  std::exit(1);
}

void check(fwant_status rc, fwant_solver* s, const char* what) {
  if (rc != FWANT_OK) die(std::string(what) + ": " + (s ? fwant_last_error(s) : "error"));
}

using seisfd::pad;

struct Snap : seisfd::SnapDef {
  std::vector<float> vbuf, tbuf;  // frames of the current file
  std::vector<float> times;
  int frames() const { return int(times.size()); }
  size_t npts() const { return size_t(subc[0]) * subc[1] * subc[2]; }
  int file_no(int ntime) const { return (ntime + tinv * tcnt - 1) / (tinv * tcnt); }
};

std::vector<float> read_f(const nc3::Reader& r, const std::string& file, const std::string& var, size_t want) {
  std::vector<float> v;
  std::string err;
  if (!r.read(var, &v, &err)) die(file + ": " + err);
  if (want && v.size() != want) die(file + ": variable " + var + " has " + std::to_string(v.size()) + " values, " +
                                    std::to_string(want) + " expected");
  return v;
}
std::vector<int> read_i(const nc3::Reader& r, const std::string& file, const std::string& var, size_t want) {
  std::vector<int> v;
  std::string err;
  if (!r.read(var, &v, &err)) die(file + ": " + err);
  if (want && v.size() != want) die(file + ": variable " + var + " has the wrong size");
  return v;
}
double att(const nc3::Reader& r, const std::string& file, const std::string& name) {
  const nc3::Att* a = r.gatt(name);
  if (!a || a->num.empty()) die(file + ": global attribute " + name + " missing");
  return a->num[0];
}

void open_nc(nc3::Reader& r, const std::string& path) {
  std::string err;
  if (!r.open(path, &err)) die(err);
}

// one vel_ or sgt_ snapshot file: dims I J K time, time(time), components (time,K,J,I)
void write_snap_file(const std::string& root, const Snap& sp, bool vel, float stept, int ntime_last) {
  if (sp.frames() == 0) return;
  nc3::Writer w;
  const int I = w.add_dim("I", sp.subc[0]), J = w.add_dim("J", sp.subc[1]), K = w.add_dim("K", sp.subc[2]);
  const int T = w.add_dim("time", 0);
  w.set_numrecs(sp.frames());
  w.add_gatt("stept", nc3::NC_FLOAT, {double(stept * float(sp.tinv))});
  w.add_gatt_text("title", vel ? "snap of velocity feilds" : "snap of stress feilds");
  std::vector<double> gs(sp.gsubs, sp.gsubs + 3), gc(sp.subc, sp.subc + 3), gt(sp.subt, sp.subt + 3),
      ge(sp.gsube, sp.gsube + 3);
  for (const char* p : {"g", ""}) {
    w.add_gatt(std::string(p) + "subs", nc3::NC_INT, gs);
    w.add_gatt(std::string(p) + "subc", nc3::NC_INT, gc);
    w.add_gatt(std::string(p) + "subt", nc3::NC_INT, gt);
    w.add_gatt(std::string(p) + "sube", nc3::NC_INT, ge);
  }
  w.add_var("time", nc3::NC_FLOAT, {T}, std::vector<double>(sp.times.begin(), sp.times.end()));
  const int nc = vel ? 3 : 6;
  const std::vector<float>& buf = vel ? sp.vbuf : sp.tbuf;
  const size_t n = sp.npts();
  static const char* const vnames[3] = {"Vx", "Vy", "Vz"};
  static const char* const tnames[6] = {"Txx", "Tyy", "Tzz", "Txy", "Txz", "Tyz"};
  for (int c = 0; c < nc; ++c) {
    std::vector<float> d(size_t(sp.frames()) * n);
    for (int f = 0; f < sp.frames(); ++f)
      std::memcpy(&d[size_t(f) * n], &buf[(size_t(f) * nc + c) * n], n * sizeof(float));
    w.add_var_f(vel ? vnames[c] : tnames[c], {T, K, J, I}, d.data(), d.size());
  }
  const std::string path = seisfd::snap_file(root, vel ? "vel_" : "sgt_", sp.id, sp.file_no(ntime_last));
  std::string err;
  if (!w.write(path, &err)) die(err);
}

// frames of a partly written snapshot group back from its file (resume)
void reload_snap_file(const std::string& root, Snap& sp, bool vel, int ntime) {
  const std::string path = seisfd::snap_file(root, vel ? "vel_" : "sgt_", sp.id, sp.file_no(ntime));
  nc3::Reader r;
  std::string err;
  if (!r.open(path, &err)) die("resume: " + err);
  const int nc = vel ? 3 : 6;
  static const char* const vnames[3] = {"Vx", "Vy", "Vz"};
  static const char* const tnames[6] = {"Txx", "Tyy", "Tzz", "Txy", "Txz", "Tyz"};
  const std::vector<float> t = read_f(r, path, "time", 0);
  const size_t n = sp.npts();
  std::vector<float>& buf = vel ? sp.vbuf : sp.tbuf;
  buf.assign(t.size() * nc * n, 0.0f);
  for (int c = 0; c < nc; ++c) {
    const std::vector<float> d = read_f(r, path, vel ? vnames[c] : tnames[c], t.size() * n);
    for (size_t f = 0; f < t.size(); ++f) std::memcpy(&buf[(f * nc + c) * n], &d[f * n], n * sizeof(float));
  }
  sp.times = t;
}

int nc_tool(int argc, char** argv) {
  const std::string mode = argv[1];
  if (argc < 3) die("usage: fwant_wave --nc-dump FILE | --nc-copy IN OUT");
  nc3::Reader r;
  open_nc(r, argv[2]);
  std::string err;
  if (mode == "--nc-dump") {
    std::printf("{\"numrecs\": %llu, \"dims\": {", (unsigned long long)r.numrecs());
    for (size_t i = 0; i < r.dims.size(); ++i)
      std::printf("%s\"%s\": %llu", i ? ", " : "", r.dims[i].name.c_str(), (unsigned long long)r.dims[i].len);
    std::printf("}, \"vars\": {");
    for (size_t i = 0; i < r.vars.size(); ++i) {
      std::vector<double> d;
      if (!r.read(r.vars[i].name, &d, &err)) die(err);
      double s = 0.0;
      for (double x : d) s += x;
      std::printf("%s\"%s\": {\"type\": %d, \"count\": %zu, \"sum\": %.17g}", i ? ", " : "", r.vars[i].name.c_str(),
                  r.vars[i].type, d.size(), s);
    }
    std::printf("}}\n");
    return 0;
  }
  if (mode == "--nc-copy" && argc >= 4) {
    nc3::Writer w;
    for (const nc3::Dim& d : r.dims) w.add_dim(d.name, d.len);
    w.set_numrecs(r.numrecs());
    for (const nc3::Att& a : r.gatts) {
      if (a.type == nc3::NC_CHAR) w.add_gatt_text(a.name, a.text);
      else w.add_gatt(a.name, a.type, a.num);
    }
    for (const nc3::Var& v : r.vars) {
      std::vector<double> d;
      if (!r.read(v.name, &d, &err)) die(err);
      w.add_var(v.name, v.type, v.dims, d);
    }
    if (!w.write(argv[3], &err)) die(err);
    return 0;
  }
  die("usage: fwant_wave --nc-dump FILE | --nc-copy IN OUT");
}

}  // namespace

// seismo_mpi000000.nc with the samples recorded up to ntime: dims num_pt,
// time(unlimited); time(time); components (time, num_pt) (io_seismo_put's file)
void write_seismo(const std::string& out_root, fwant_solver* s, int ntime, int pt_tinv, int num_pt, float fstept) {
  int nsamp = ntime / pt_tinv;
  std::vector<float> seis(size_t(9) * nsamp * num_pt);
  check(fwant_get_seismo(s, seis.data(), nsamp, &nsamp), s, "seismograms");
  nc3::Writer w;
  const int P = w.add_dim("num_pt", num_pt), T = w.add_dim("time", 0);
  w.set_numrecs(nsamp);
  w.add_gatt_text("title", "seismograms");
  std::vector<double> t(nsamp);
  for (int m = 0; m < nsamp; ++m) t[m] = double(float((m + 1) * pt_tinv) * fstept);  // t = ntime*stept
  w.add_var("time", nc3::NC_FLOAT, {T}, t);
  for (int c = 0; c < 9; ++c)
    w.add_var_f(COMP[c], {T, P}, seis.data() + size_t(c) * nsamp * num_pt, size_t(nsamp) * num_pt);
  std::string err;
  if (!w.write(out_root + "/seismo_" + SUFFIX + ".nc", &err)) die(err);
}

// The run-time log (swmpi_time_init / _write / _end, code/srcF/mod_mpi.F90:331-405): a
// header, then one line per step with its wall time, the hours passed and the hours left.
// Steps run in graph-replayed chunks between output events, so each step of a chunk is
// logged with the chunk's average time.
class StepLog {
 public:
  StepLog(const std::string& path, int ntime) : path_(path), n0_(ntime) {
    if (path_.empty()) return;
    t0_ = t1_ = now();
    std::FILE* f = std::fopen(path_.c_str(), ntime == 0 ? "w" : "a");
    if (!f) die("cannot open the run-time log " + path_);
    if (ntime == 0) std::fprintf(f, " # seis3d_wave run time log\n");
    else std::fprintf(f, "\n # seis3d_wave restart from ntime= %d\n", ntime);
    std::fprintf(f, "\n the program begins from %s\n\n each step uses time\n", stamp().c_str());
    std::fclose(f);
  }
  void steps(int from, int to, int total) {
    if (path_.empty() || to <= from) return;
    const double t2 = now(), per = (t2 - t1_) / double(to - from);
    std::FILE* f = std::fopen(path_.c_str(), "a");
    if (!f) return;
    for (int n = from + 1; n <= to; ++n) {
      const double passed = (t1_ + per * (n - from) - t0_) / 3600.0;
      const double left = passed / double(n - n0_) * double(total - n0_) - passed;
      std::fprintf(f, "%6d step uses%12.5G s,  %12.5G hours passed and%12.5G hours left\n", n, per, passed, left);
    }
    std::fclose(f);
    t1_ = t2;
  }
  void end() {
    if (path_.empty()) return;
    const double sec = now() - t0_;
    const int d = int(sec / 86400.0), h = int((sec - d * 86400.0) / 3600.0), m = int((sec - d * 86400.0 - h * 3600.0) / 60.0);
    std::FILE* f = std::fopen(path_.c_str(), "a");
    if (!f) return;
    std::fprintf(f, " ------------------------------------\n the program\n   finish at %s\n the total run time is\n"
                 "%10d       day%10d      hour%10d    minute\n", stamp().c_str(), d, h, m);
    std::fclose(f);
  }

 private:
  static double now() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
  }
  static std::string stamp() {
    const std::time_t t = std::time(nullptr);
    char b[64];
    std::strftime(b, sizeof(b), "%Y%m%d,%H/%M/%S", std::localtime(&t));
    return b;
  }
  std::string path_;
  int n0_ = 0;
  double t0_ = 0.0, t1_ = 0.0;
};

int main(int argc, char** argv) {
  if (argc >= 2 && std::strncmp(argv[1], "--nc-", 5) == 0) return nc_tool(argc, argv);
  std::string conf_path = "SeisFD3D.conf";
  int device = 0, storage = FWANT_STORAGE_FP32, exact = 0;
  for (int a = 1; a < argc; ++a) {
    const std::string s = argv[a];
    if (s == "--device" && a + 1 < argc) device = std::atoi(argv[++a]);
    else if (s == "--storage" && a + 1 < argc) {
      const std::string v = argv[++a];
      storage = v == "bf16" ? FWANT_STORAGE_BF16 : v == "fp16" ? FWANT_STORAGE_FP16 : FWANT_STORAGE_FP32;
    } else if (s == "--exact") exact = 1;
    else conf_path = s;
  }
  conf::File cf;
  std::string err;
  if (!cf.load(conf_path, &err)) die(err);
  auto need_i = [&](const std::string& k, int col) {
    int v;
    if (!cf.get_int(k, col, &v)) die(conf_path + ": key " + k + " column " + std::to_string(col) + " missing");
    return v;
  };
  auto need_d = [&](const std::string& k, int col) {
    double v;
    if (!cf.get_double(k, col, &v)) die(conf_path + ": key " + k + " column " + std::to_string(col) + " missing");
    return v;
  };
  auto need_s = [&](const std::string& k) {
    std::string v;
    if (!cf.get(k, 2, &v)) die(conf_path + ": key " + k + " missing");
    return v;
  };
  // para_init (code/srcF/mod_para.F90:70-88)
  const int ni = need_i("ni", 2), nj = need_i("nj", 2), nk = need_i("nk", 2), nt = need_i("nt", 2);
  const double stept = need_d("stept", 2);
  if (cf.has("dims"))
    for (int d = 0; d < 3; ++d)
      if (need_i("dims", d + 2) != 1) die("dims must be 1 1 1: one GPU runs the whole grid (fwant_prep stitch turns a multi-rank input set into one rank)");
  const std::string grid_root = need_s("GRID_ROOT"), media_root = need_s("MEDIA_ROOT"),
                    source_root = need_s("SOURCE_ROOT"), station_root = need_s("STATION_ROOT"),
                    out_root = need_s("OUTPUT_ROOT");
  std::string ckpt_root;
  int ckpt_tinv = 0, from_ckpt = 0;
  if (cf.has("CHECKPOINT_ROOT")) ckpt_root = need_s("CHECKPOINT_ROOT");
  if (cf.has("checkpoint_tinv")) ckpt_tinv = need_i("checkpoint_tinv", 2);
  if (cf.has("run_from_checkpoint")) from_ckpt = need_i("run_from_checkpoint", 2);
  // io_init (code/srcF/mod_io.F90:98-106): the urgent-checkpoint control file and the
  // per-step run-time log, both optional here
  std::string urgent_path, log_path;
  if (cf.has("urgent_checkpoint")) urgent_path = need_s("urgent_checkpoint");
  if (cf.has("fnm_log")) log_path = need_s("fnm_log");
  // abs_init keys (code/srcF/mod_abs_npml.F90:157-178), columns x1 x2 y1 y2 z1 z2
  int pml_n[6];
  float pml_v[6], pml_b[6], pml_a[6];
  for (int f = 0; f < 6; ++f) {
    pml_n[f] = need_i("abs_number", f + 2);
    pml_v[f] = pml_n[f] > 0 ? float(need_d("abs_velocity", f + 2)) : 0.0f;
    pml_b[f] = pml_n[f] > 0 ? float(need_d("CFS_bmax", f + 2)) : 1.0f;
    pml_a[f] = pml_n[f] > 0 ? float(need_d("CFS_amax", f + 2)) : 0.0f;
  }
  const int nx = ni + 6, ny = nj + 6, nz = nk + 6;
  const size_t n3 = size_t(nx) * ny * nz;

  // inputs (grid_coord_import, grid_metric_import, media_import, src_import, io_pt_import)
  nc3::Reader fc, fm, fmed, fsrc, fsta;
  const std::string pc = grid_root + "/coord_" + SUFFIX + ".nc", pm = grid_root + "/metric_" + SUFFIX + ".nc",
                    pmed = media_root + "/media_" + SUFFIX + ".nc", psrc = source_root + "/source_" + SUFFIX + ".nc",
                    psta = station_root + "/station_" + SUFFIX + ".nc";
  open_nc(fc, pc);
  open_nc(fm, pm);
  open_nc(fmed, pmed);
  open_nc(fsrc, psrc);
  open_nc(fsta, psta);

  fwant_config cfg{};
  cfg.ni = ni; cfg.nj = nj; cfg.nk = nk; cfg.stept = stept;
  cfg.free_surface = pml_n[5] > 0 ? 0 : 1;
  cfg.src_surface = 1;
  cfg.storage = storage;
  cfg.device = device;
  cfg.exact_arith = exact;
  fwant_solver* s = nullptr;
  check(fwant_create(&cfg, &s), nullptr, "create");
  {
    const auto x = read_f(fc, pc, "x", nx), y = read_f(fc, pc, "y", ny), z = read_f(fc, pc, "z", nz);
    check(fwant_set_coord(s, x.data(), y.data(), z.data()), s, "coordinates");
    const auto a = read_f(fm, pm, "xsin", nx), b = read_f(fm, pm, "xcot", nx), c = read_f(fm, pm, "xi_x", nx),
               d = read_f(fm, pm, "eta_y", ny), e = read_f(fm, pm, "zeta_z", nz);
    check(fwant_set_metric(s, a.data(), b.data(), c.data(), d.data(), e.data()), s, "metric");
    const auto lam = read_f(fmed, pmed, "lambda", n3), mu = read_f(fmed, pmed, "mu", n3),
               rho = read_f(fmed, pmed, "rho", n3);
    check(fwant_set_media(s, lam.data(), mu.data(), rho.data()), s, "media");
  }
  check(fwant_set_pml(s, pml_n, pml_v, pml_b, pml_a), s, "PML");
  const int nforce = int(att(fsrc, psrc, "number_of_force")), nmom = int(att(fsrc, psrc, "number_of_moment"));
  if (nforce > 0) {
    const nc3::Dim* tw = fsrc.dim("force_time_window");
    if (!tw) die(psrc + ": dimension force_time_window missing");
    const int ntw = int(tw->len);
    const auto indx = read_i(fsrc, psrc, "force_indx", size_t(3) * nforce);
    const auto shift = read_f(fsrc, psrc, "force_shift", size_t(3) * nforce);
    const auto t0 = read_f(fsrc, psrc, "force_start_time", nforce);
    const auto st = read_f(fsrc, psrc, "force_stf_time", ntw), sf = read_f(fsrc, psrc, "force_stf_freq", ntw);
    const auto fx = read_f(fsrc, psrc, "Fx", size_t(ntw) * nforce), fy = read_f(fsrc, psrc, "Fy", size_t(ntw) * nforce),
               fz = read_f(fsrc, psrc, "Fz", size_t(ntw) * nforce);
    check(fwant_set_forces(s, nforce, ntw, indx.data(), shift.data(), t0.data(), st.data(), sf.data(), fx.data(),
                           fy.data(), fz.data(), int(att(fsrc, psrc, "force_stf_id"))),
          s, "forces");
  }
  if (nmom > 0) {
    const nc3::Dim* tw = fsrc.dim("moment_time_window");
    if (!tw) die(psrc + ": dimension moment_time_window missing");
    const int ntw = int(tw->len);
    const auto indx = read_i(fsrc, psrc, "moment_indx", size_t(3) * nmom);
    const auto shift = read_f(fsrc, psrc, "moment_shift", size_t(3) * nmom);
    const auto t0 = read_f(fsrc, psrc, "moment_start_time", nmom);
    const auto st = read_f(fsrc, psrc, "moment_stf_time", ntw), sf = read_f(fsrc, psrc, "moment_stf_freq", ntw);
    std::vector<float> mom;
    for (const char* nm : {"Mxx", "Myy", "Mzz", "Mxy", "Mxz", "Myz"}) {
      const auto m = read_f(fsrc, psrc, nm, size_t(ntw) * nmom);
      mom.insert(mom.end(), m.begin(), m.end());
    }
    check(fwant_set_moments(s, nmom, ntw, indx.data(), shift.data(), t0.data(), st.data(), sf.data(), mom.data(),
                            int(att(fsrc, psrc, "moment_stf_id"))),
          s, "moments");
  }
  const nc3::Dim* npd = fsta.dim("num_pt");
  if (!npd) die(psta + ": dimension num_pt missing");
  const int num_pt = int(npd->len == 0 ? fsta.numrecs() : npd->len);
  const int pt_tinv = int(att(fsta, psta, "tinv"));
  if (num_pt > 0) {
    const auto indx = read_i(fsta, psta, "indx", size_t(3) * num_pt);
    check(fwant_set_receivers(s, num_pt, indx.data(), pt_tinv), s, "receivers");
  }
  // snapshots (io_snap_read / corr_indx / io_snap_locate, code/srcF/mod_io.F90:180-262)
  std::vector<Snap> snaps;
  try {
    for (const seisfd::SnapDef& d : seisfd::read_snaps(cf, ni, nj, nk)) {
      Snap sp;
      static_cast<seisfd::SnapDef&>(sp) = d;
      snaps.push_back(sp);
    }
  } catch (const std::exception& e) {
    die(conf_path + ": " + e.what());
  }

  const int total = fwant_reference_steps(nt);
  int ntime = 0;
  if (from_ckpt > 0) {
    const std::string path = ckpt_root + "/rest_t" + pad(from_ckpt, 5) + "_" + SUFFIX + ".ckpt";
    check(fwant_load_checkpoint(s, path.c_str()), s, "resume");
    check(fwant_get_ntime(s, &ntime), s, "resume");
    for (Snap& sp : snaps)
      if ((ntime / sp.tinv) % sp.tcnt != 0) {
        if (sp.vel) reload_snap_file(out_root, sp, true, ntime);
        if (sp.sgt) reload_snap_file(out_root, sp, false, ntime);
      }
  }
  std::string prev_ckpt;
  const float fstept = float(stept);
  StepLog steplog(log_path, ntime);
  int nt_dyn_rest = 0, nt_dyn_sync = 0;
  int total_now = total;
  while (ntime < total_now) {
    // next step at which something is written or read
    int next = total_now;
    for (const Snap& sp : snaps) next = std::min(next, (ntime / sp.tinv + 1) * sp.tinv);
    if (ckpt_tinv > 0) next = std::min(next, (ntime / ckpt_tinv + 1) * ckpt_tinv);
    if (!urgent_path.empty()) next = std::min(next, (ntime / 10 + 1) * 10);
    if (nt_dyn_rest > ntime) next = std::min(next, nt_dyn_rest);
    if (nt_dyn_sync > ntime) next = std::min(next, nt_dyn_sync);
    check(fwant_run(s, next - ntime), s, "run");
    steplog.steps(ntime, next, total_now);
    ntime = next;
    for (Snap& sp : snaps) {
      if (ntime % sp.tinv != 0) continue;
      const size_t n = sp.npts();
      std::vector<float> frame;
      if (sp.vel) {
        const int comps[3] = {0, 1, 2};
        frame.resize(3 * n);
        check(fwant_get_snapshot(s, sp.subs, sp.subc, sp.subt, 3, comps, frame.data()), s, "snapshot");
        sp.vbuf.insert(sp.vbuf.end(), frame.begin(), frame.end());
      }
      if (sp.sgt) {
        const int comps[6] = {3, 4, 5, 6, 7, 8};
        frame.resize(6 * n);
        check(fwant_get_snapshot(s, sp.subs, sp.subc, sp.subt, 6, comps, frame.data()), s, "snapshot");
        sp.tbuf.insert(sp.tbuf.end(), frame.begin(), frame.end());
      }
      sp.times.push_back(float(ntime) * fstept);
      if (sp.frames() == sp.tcnt) {
        if (sp.vel) write_snap_file(out_root, sp, true, fstept, ntime);
        if (sp.sgt) write_snap_file(out_root, sp, false, fstept, ntime);
        sp.vbuf.clear(); sp.tbuf.clear(); sp.times.clear();
      }
    }
    // the urgent-checkpoint file, re-read every 10 steps (io_rest_export :350-362): a
    // checkpoint step, a sync step and a new nt (taken when it lies ahead)
    if (!urgent_path.empty() && ntime % 10 == 0) {
      std::ifstream uf(urgent_path);
      int r = 0, y = 0, nw = 0;
      if (!uf || !(uf >> r >> y >> nw)) die("io_rest_export: error when open " + urgent_path);
      nt_dyn_rest = r;
      nt_dyn_sync = y;
      if (nw > ntime) {
        std::printf("reset nt to %d step\n", nw);
        total_now = fwant_reference_steps(nw);
      }
    }
    const bool rest_now = (ckpt_tinv > 0 && ntime % ckpt_tinv == 0) || ntime == nt_dyn_rest;
    if ((rest_now || ntime == nt_dyn_sync) && ntime < total_now && num_pt > 0) {
      // nf90_sync: the seismograms so far are on disk
      write_seismo(out_root, s, ntime, pt_tinv, num_pt, fstept);
    }
    if (rest_now && ntime < total_now) {
      // partly filled snapshot groups go to their files so that a resume can read them back
      for (Snap& sp : snaps) {
        if (sp.vel) write_snap_file(out_root, sp, true, fstept, ntime);
        if (sp.sgt) write_snap_file(out_root, sp, false, fstept, ntime);
      }
      const std::string path = ckpt_root + "/rest_t" + pad(ntime, 5) + "_" + SUFFIX + ".ckpt";
      check(fwant_save_checkpoint(s, path.c_str()), s, "checkpoint");
      if (!prev_ckpt.empty()) std::remove(prev_ckpt.c_str());  // the reference keeps one restart
      prev_ckpt = path;
    }
  }
  for (Snap& sp : snaps) {  // groups the run ended in
    if (sp.vel) write_snap_file(out_root, sp, true, fstept, ntime);
    if (sp.sgt) write_snap_file(out_root, sp, false, fstept, ntime);
  }
  if (num_pt > 0) write_seismo(out_root, s, ntime, pt_tinv, num_pt, fstept);
  steplog.end();
  double ms = 0.0;
  fwant_last_run_ms(s, &ms);
  std::printf("fwant_wave: %d steps of %dx%dx%d, %d receivers, %zu snapshot series\n", ntime, ni, nj, nk, num_pt,
              snaps.size());
  fwant_destroy(s);
  return 0;
}
