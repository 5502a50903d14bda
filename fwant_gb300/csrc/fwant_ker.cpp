// fwant_ker — the station sensitivity-kernel program (SI_ker_sta,
// code/srcF.kernel/SI_ker_sta.F90) over the C ABI, one rank on one GPU.
//
// Inputs as the reference reads them: TomoKernel.conf (init_kernel :1047-1082, filter list
// init_filter :1084-1112) naming the solver's SeisFD3D.conf (grid, time step, snapshot
// series, MEDIA_ROOT); on standard input the station list file and the rank id (0 0 0);
// the station list gives per station an event list; an event list holds per event a header
// line (name, six pick counts, the 3x3 rotation matrix column by column), three synthetic
// files (T V U per line) and the pick lines (frequency band, P1 / P2 / N, t1, t2, output
// directory).  Strain Green's tensors come from the sgt_ snapshot files of the station's
// three force runs (SGT_ROOT/<station>/SGT_STA{X,Y,Z}) and of the event run
// (EVENT_ROOT/<event>/EVENT_OUTD), read block by block as strided sub-volumes.
//
// Per block (:179-345) and event: the scatter series of the flagged force components
// (stress2strain + sgt2scatter3 on the device, FP64 sums), the component rotation at the
// first rotated component (syn_rotate of V, U in single precision on the host as the
// reference does; scatter_rotate on the device), then per pick the window (:676-704), the
// filter of the pick's band (:756-773) and the window kernels, written into
// <pick directory>/kernel_NNN_mpi000000_n00000.nc (phase_Vp amplitude_Vp phase_Vs
// amplitude_Vs over the snapshot's I J K), created at the first block of a first run and
// updated in place by the later blocks.  With --lamu the program is SI_ker_sta_lamu: the
// lambda/mu kernels (SI_ker_sta_lamu.F90:1299-1300) into kernel_lamu_NNN_mpi000000_n00000.nc
// (phase_la amplitude_la phase_mu amplitude_mu); everything else is the same.
//
// With --convert MODE the program is one of the kernel conversions, which walk the same
// stations, blocks, events and picks (TomoKernel_conv.conf by default; on standard input the
// input directory, the station list file, the rank id) but read each pick's kernel file
// <input directory><pick directory>/<input file> block by block instead of forming it from
// SGTs, convert it point by point with the block's lambda and mu on the device, and write
// <pick directory>/<output file>:
//   lamu2kamu  SI_ker_lamu2kamu: kernel_lamu_ (la, mu) -> kernel_ (kappa, mu, under the
//              Vp/Vs variable names the reference gives them)
//   lamu2vpvs  SI_ker_lamu2vpvs: kernel_lamu_ (la, mu) -> kernel_ (Vp, Vs)
//   vpvs2kamu  SI_ker_vpvs2kamu: kernel_ (Vp, Vs) -> kernel_kamu_ (phase_ka amplitude_ka
//              phase_mu amplitude_mu)
// The time axis is T(n) = n kdt (SI_ker_lamu2kamu.F90:260-263): the synthetics are listed
// but not read, and a pick whose window lies outside it is skipped as in the kernel run.
//
// With --eq the program is SI_ker_EQ (code/srcF.kernel/SI_ker_EQ.F90): SI_ker_sta with the
// station's Z-force SGT moved 9 frames earlier in time, the last 9 frames zero
// (eoshift(., shift=9) along time, SI_ker_EQ.F90:580-586); everything else is the same.
//
// Tool modes (format checks): --nc-slab FILE VAR START COUNT STRIDE prints a strided
// sub-array as JSON; --nc-fill-slab FILE VAR START COUNT STRIDE writes 1, 2, ... into one
// (comma-separated lists, slowest dimension first, 0-based starts).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/fwant_gb300.h"
#include "../../include/fwant_kerinfo.h"
#include "conf.h"
#include "netcdf3.h"
#include "seisfd_conf.h"

namespace {

[[noreturn]] void die(const std::string& msg) {
  std::fprintf(stderr, "fwant_ker: %s\n", msg.c_str());
  std::exit(1);
}

void check(fwant_status rc, fwant_sgtker* k, const char* what) {
  if (rc != FWANT_OK) die(std::string(what) + ": " + (k ? fwant_sgtker_last_error(k) : "error"));
}

std::vector<std::string> words(const std::string& line) {
  std::vector<std::string> w;
  std::istringstream is(line);
  for (std::string s; is >> s;) w.push_back(s);
  return w;
}

std::string unquote(std::string s) {
  if (s.size() >= 2 && (s[0] == '\'' || s[0] == '"') && s.back() == s[0]) s = s.substr(1, s.size() - 2);
  return s;
}

std::string trim(const std::string& s) {
  const size_t a = s.find_first_not_of(" \t\r\n");
  if (a == std::string::npos) return "";
  const size_t b = s.find_last_not_of(" \t\r\n");
  return s.substr(a, b - a + 1);
}

// list-directed logical: optional '.', then T/t or F/f
bool parse_logical(const std::string& s, const std::string& key) {
  size_t i = 0;
  while (i < s.size() && s[i] == '.') ++i;
  if (i < s.size() && (s[i] == 'T' || s[i] == 't')) return true;
  if (i < s.size() && (s[i] == 'F' || s[i] == 'f')) return false;
  die("key " + key + ": not a logical value: " + s);
}

float to_f(const std::string& s, const std::string& what) {
  char* end = nullptr;
  std::string t = s;
  for (char& c : t)
    if (c == 'd' || c == 'D') c = 'e';  // Fortran double-precision exponent
  const double v = std::strtod(t.c_str(), &end);
  if (end == t.c_str()) die(what + ": not a number: " + s);
  return float(v);
}
int to_i(const std::string& s, const std::string& what) {
  char* end = nullptr;
  const long v = std::strtol(s.c_str(), &end, 10);
  if (end == s.c_str()) die(what + ": not an integer: " + s);
  return int(v);
}

// A Fortran F20.16 input field: blanks ignored, no decimal point means 16 implied digits.
double fixed_field(const std::string& f) {
  std::string t;
  for (char c : f)
    if (c != ' ' && c != '\t' && c != '\r' && c != '\n') t.push_back(c == 'd' || c == 'D' ? 'e' : c);
  if (t.empty()) return 0.0;
  const double v = std::strtod(t.c_str(), nullptr);
  const bool has_point = t.find('.') != std::string::npos;
  const bool has_exp = t.find_first_of("eE") != std::string::npos;
  return (has_point || has_exp) ? v : v * 1e-16;
}

struct Filter {  // one frequency band's coefficients (a(1..nod1), b(1..nod1)); none: nod1 = 0
  int nod1 = 0;
  std::vector<double> a, b;
};

// <filter_file> followed by num_freq file names (init_filter, SI_ker_sta.F90:1084-1112):
// each file holds NOD1, then NOD1 lines "(2(f20.16))" of a and b.
std::vector<Filter> read_filters(const std::string& conf_path, int num_freq) {
  std::ifstream in(conf_path);
  if (!in) die("cannot open " + conf_path);
  std::string line;
  bool found = false;
  while (std::getline(in, line)) {
    std::string t = line.substr(0, line.find('#'));
    for (char& c : t)
      if (c == '=' || c == '\t' || c == '|') c = ' ';
    const auto w = words(t);
    if (!w.empty() && w[0] == "<filter_file>") { found = true; break; }
  }
  if (!found) die(conf_path + ": <filter_file> missing");
  std::vector<Filter> out(size_t(std::max(num_freq, 0)));
  for (int n = 0; n < num_freq; ++n) {
    std::vector<std::string> w;
    while (w.empty()) {
      if (!std::getline(in, line)) die(conf_path + ": fewer filter files than number_of_freqband");
      w = words(line);
    }
    const std::string name = unquote(w[0]);
    if (name == "none") continue;
    std::ifstream f(name);
    if (!f) die("cannot open filter file " + name);
    std::string l;
    std::vector<std::string> hw;
    while (hw.empty() && std::getline(f, l)) hw = words(l);
    if (hw.empty()) die(name + ": order missing");
    const int nod1 = to_i(hw[0], name);
    if (nod1 < 1) die(name + ": NOD1 must be >= 1");
    Filter& F = out[size_t(n)];
    F.nod1 = nod1;
    for (int m = 0; m < nod1; ++m) {
      if (!std::getline(f, l)) die(name + ": fewer coefficient lines than NOD1");
      l.resize(std::max<size_t>(l.size(), 40), ' ');
      F.a.push_back(fixed_field(l.substr(0, 20)));
      F.b.push_back(fixed_field(l.substr(20, 20)));
    }
  }
  return out;
}

struct Pick {
  int freq = 0, filt = 0;  // filt: 0 none, 1 one-pass, 2 forward-backward
  float t1 = 0, t2 = 0;
  std::string dir;
};

struct Event {
  std::string name;
  int picknum[6] = {0, 0, 0, 0, 0, 0};
  float rot[9];                        // rot_mat column by column
  std::string syn[3];
  std::vector<Pick> picks[6];
};

// One event list (SI_ker_sta.F90:350-400, 650-715): comment lines start with '#'.
// strict false: SI_ker2info's reading (SI_ker2info.F90:193-262), which takes the pick's
// band and filter name as they stand.
std::vector<Event> read_events(const std::string& path, int num_freq, bool strict = true) {
  std::ifstream in(path);
  if (!in) die("evt_list open err: " + path);
  std::vector<Event> out;
  std::string line;
  auto next_line = [&](bool skip_comments, const char* what) {
    for (;;) {
      if (!std::getline(in, line)) die(path + ": " + what + " missing");
      const std::string t = trim(line);
      if (skip_comments && !t.empty() && t[0] == '#') continue;
      return t;
    }
  };
  while (std::getline(in, line)) {
    const std::string t = trim(line);
    if (t.empty() || t[0] == '#') continue;
    const auto w = words(t);
    if (w.size() < 16) die(path + ": event line needs a name, 6 pick counts and 9 matrix entries: " + t);
    Event e;
    e.name = w[0];
    for (int c = 0; c < 6; ++c) e.picknum[c] = to_i(w[1 + c], path);
    for (int q = 0; q < 9; ++q) e.rot[q] = to_f(w[7 + q], path);
    for (int c = 0; c < 3; ++c) e.syn[c] = trim(next_line(false, "synthetic file name"));
    bool any = false;
    for (int c = 0; c < 6; ++c) any = any || e.picknum[c] > 0;
    if (any)
      for (int c = 0; c < 6; ++c)
        for (int p = 0; p < e.picknum[c]; ++p) {
          const std::string pl = next_line(true, "pick line");
          const auto pw = words(pl);
          if (pw.size() < 5) die(path + ": pick line needs band, filter, t1, t2 and a directory: " + pl);
          Pick pk;
          pk.freq = to_i(pw[0], path);
          if (strict && pk.freq > num_freq) die("frequency band id overflow");
          if (pw[1] == "P1") pk.filt = 1;
          else if (pw[1] == "P2") pk.filt = 2;
          else if (pw[1] == "N" || !strict) pk.filt = 0;
          else die(path + ": pickfilt error: " + pw[1]);
          pk.t1 = to_f(pw[2], path);
          pk.t2 = to_f(pw[3], path);
          // the rest of the line after t2 is the output directory
          size_t pos = 0;
          for (int k = 0; k < 4; ++k) {
            pos = pl.find_first_not_of(" \t", pos);
            pos = pl.find_first_of(" \t", pos);
          }
          pk.dir = trim(pl.substr(pos == std::string::npos ? pl.size() : pos));
          e.picks[c].push_back(pk);
        }
    out.push_back(e);
  }
  return out;
}

// knt lines of T V U (init_synthetic, SI_ker_sta.F90:1114-1125)
void read_synthetic(const std::string& path, int knt, std::vector<float>& T, std::vector<float>& V,
                    std::vector<float>& U) {
  std::ifstream in(path);
  if (!in) die("cannot open synthetic file " + path);
  T.resize(size_t(knt));
  V.resize(size_t(knt));
  U.resize(size_t(knt));
  std::string tok;
  auto num = [&]() {
    if (!(in >> tok)) die(path + ": fewer than SGT_TIMEDIM_SIZE samples");
    return to_f(tok, path);
  };
  for (int n = 0; n < knt; ++n) {
    T[size_t(n)] = num();
    V[size_t(n)] = num();
    U[size_t(n)] = num();
  }
}

// syn_rotate (SI_ker_sta.F90:1339-1352) in single precision, operands in the reference's order
void syn_rotate(std::vector<float>* v, const float* r) {
  for (size_t n = 0; n < v[0].size(); ++n) {
    const float v1 = v[0][n], v2 = v[1][n], v3 = v[2][n];
    for (int c = 0; c < 3; ++c) v[c][n] = (v1 * r[0 + 3 * c] + v2 * r[1 + 3 * c]) + v3 * r[2 + 3 * c];
  }
}

struct Geometry {
  int bsubs[3], bsubc[3], bsubt[3];  // block in the snapshot's sample grid (1-based)
  int subs[3], subt[3];              // the same points in the grid with ghosts (media file)
  size_t npts() const { return size_t(bsubc[0]) * bsubc[1] * bsubc[2]; }
};

// Strided sub-array of the six stresses of one SGT series (sgt_ files of one run) for the
// block, knt frames over as many files as the series needs (SI_ker_sta.F90:406-458):
// out is (6, knt, points) with i fastest.
void read_sgt(const std::string& root, const seisfd::SnapDef& sp, const Geometry& g, int knt,
              std::vector<float>& out) {
  static const char* const names[6] = {"Txx", "Tyy", "Tzz", "Txy", "Txz", "Tyz"};
  const size_t np = g.npts();
  out.assign(6 * size_t(knt) * np, 0.0f);
  int m = 0, n = 0, mt = std::min(sp.tcnt, knt);
  std::vector<float> slab;
  while (m < knt) {
    ++n;
    const std::string path = seisfd::snap_file(root, "sgt_", sp.id, n);
    nc3::Reader r;
    std::string err;
    if (!r.open(path, &err)) die(err);
    if (m + mt > knt) mt = knt - m;
    const std::vector<uint64_t> start = {0, uint64_t(g.bsubs[2] - 1), uint64_t(g.bsubs[1] - 1), uint64_t(g.bsubs[0] - 1)};
    const std::vector<uint64_t> cnt = {uint64_t(mt), uint64_t(g.bsubc[2]), uint64_t(g.bsubc[1]), uint64_t(g.bsubc[0])};
    const std::vector<uint64_t> str = {1, uint64_t(g.bsubt[2]), uint64_t(g.bsubt[1]), uint64_t(g.bsubt[0])};
    for (int q = 0; q < 6; ++q) {
      if (!r.read_slab(names[q], start, cnt, str, &slab, &err)) die(path + ": " + err);
      std::copy(slab.begin(), slab.end(), out.begin() + ptrdiff_t((size_t(q) * knt + size_t(m)) * np));
    }
    m += mt;
  }
}

// SI_ker_EQ's shift of the station's Z-force SGT: frame n takes frame n + shift, the last
// `shift` frames 0 (eoshift along time; SI_ker_EQ.F90:580-586).  s is (6, knt, np).
constexpr int EQ_SHIFT = 9;
void shift_frames(std::vector<float>& s, int knt, size_t np, int shift) {
  for (int q = 0; q < 6; ++q)
    for (int n = 0; n < knt; ++n) {
      float* dst = s.data() + (size_t(q) * knt + size_t(n)) * np;
      if (n + shift < knt) std::copy_n(s.data() + (size_t(q) * knt + size_t(n + shift)) * np, np, dst);
      else std::fill_n(dst, np, 0.0f);
    }
}

int nc_tool(int argc, char** argv) {
  const std::string mode = argv[1];
  if (argc < 7) die("usage: " + mode + " FILE VAR START COUNT STRIDE");
  auto list = [](const std::string& s) {
    std::vector<uint64_t> v;
    std::stringstream ss(s);
    for (std::string t; std::getline(ss, t, ',');) v.push_back(std::strtoull(t.c_str(), nullptr, 10));
    return v;
  };
  const auto start = list(argv[4]), cnt = list(argv[5]), str = list(argv[6]);
  std::string err;
  if (mode == "--nc-slab") {
    nc3::Reader r;
    std::vector<float> v;
    if (!r.open(argv[2], &err) || !r.read_slab(argv[3], start, cnt, str, &v, &err)) die(err);
    std::printf("[");
    for (size_t i = 0; i < v.size(); ++i) std::printf("%s%.9g", i ? ", " : "", double(v[i]));
    std::printf("]\n");
    return 0;
  }
  if (mode == "--nc-fill-slab") {
    uint64_t n = 1;
    for (uint64_t c : cnt) n *= c;
    std::vector<float> v(static_cast<size_t>(n));
    for (size_t i = 0; i < v.size(); ++i) v[i] = float(i + 1);
    if (!nc3::update_slab(argv[2], argv[3], start, cnt, str, v.data(), &err)) die(err);
    return 0;
  }
  die("unknown tool mode " + mode);
}

// Window indices of a pick over T(n) = n kdt (maxloc(T, T <= t1), minloc(T, T >= t2);
// SI_ker_sta.F90:676-704); false (with the reference's warning) when the pick is skipped.
bool pick_window(const Pick& pk, const std::vector<float>& T, float tmin, float tmax, int* nt1, int* nt2) {
  const int knt = int(T.size());
  *nt1 = 0;
  *nt2 = 0;
  if (pk.t1 > tmax) {
    std::fprintf(stderr, "fwant_ker: t1>Tmax, skip this rcd %s\n", pk.dir.c_str());
    return false;
  } else if (pk.t1 <= tmin) {
    *nt1 = 1;
  } else {
    for (int n = 1; n <= knt; ++n)
      if (T[size_t(n - 1)] <= pk.t1 && (*nt1 == 0 || T[size_t(n - 1)] > T[size_t(*nt1 - 1)])) *nt1 = n;
  }
  if (pk.t2 < tmin) {
    std::fprintf(stderr, "fwant_ker: t2<Tmin, skip this rcd %s\n", pk.dir.c_str());
    return false;
  } else if (pk.t2 >= tmax) {
    *nt2 = knt;
  } else {
    for (int n = 1; n <= knt; ++n)
      if (T[size_t(n - 1)] >= pk.t2 && (*nt2 == 0 || T[size_t(n - 1)] < T[size_t(*nt2 - 1)])) *nt2 = n;
  }
  if (*nt1 < 1 || *nt2 < 1 || *nt1 > *nt2) die("window of pick " + pk.dir + " selects no sample");
  return true;
}

// One block of the conversion programs (SI_ker_lamu2kamu.F90:346-836 and its two siblings):
// every pick of every event, in the kernel run's order, has its input kernel block read,
// converted on the device with the block's lambda and mu (already in K) and written into
// its output file, which the first block of a first run creates.  Returns the picks done.
long long convert_block(fwant_sgtker* K, int conv, const std::vector<Event>& events, const Geometry& g,
                        const seisfd::SnapDef& sp, int kid, int knt, float kdt, float tmin, float tmax, bool create,
                        const std::string& indir, const std::string& iprefix, const char* const* iname,
                        const std::string& oprefix, const char* const* oname) {
  std::vector<float> T(static_cast<size_t>(knt));
  for (int n = 0; n < knt; ++n) T[size_t(n)] = float(n + 1) * kdt;  // T = (/1:knt/)*kdt
  const size_t np = g.npts();
  const std::vector<uint64_t> st = {uint64_t(g.bsubs[2] - 1), uint64_t(g.bsubs[1] - 1), uint64_t(g.bsubs[0] - 1)};
  const std::vector<uint64_t> ct = {uint64_t(g.bsubc[2]), uint64_t(g.bsubc[1]), uint64_t(g.bsubc[0])};
  const std::vector<uint64_t> sd = {uint64_t(g.bsubt[2]), uint64_t(g.bsubt[1]), uint64_t(g.bsubt[0])};
  const std::string fname = seisfd::pad(kid, 3) + "_" + seisfd::MPI_SUFFIX + "_n00000.nc";
  long long done = 0;
  std::string err;
  for (const Event& e : events) {
    bool any = false;
    for (int c = 0; c < 6; ++c) any = any || e.picknum[c] > 0;
    if (!any) continue;
    for (int ncmp = 1; ncmp <= 6; ++ncmp)
      for (const Pick& pk : e.picks[ncmp - 1]) {
        int nt1, nt2;
        if (!pick_window(pk, T, tmin, tmax, &nt1, &nt2)) continue;
        const std::string out = pk.dir + oprefix + fname;
        if (create) {  // nfseis_grid3d_def over the snapshot's points
          nc3::Writer wr;
          const int di = wr.add_dim("I", uint64_t(sp.subc[0])), dj = wr.add_dim("J", uint64_t(sp.subc[1])),
                    dk = wr.add_dim("K", uint64_t(sp.subc[2]));
          wr.add_gatt_text("title", "Finite frequency kernel");
          const size_t n3 = size_t(sp.subc[0]) * sp.subc[1] * sp.subc[2];
          const std::vector<float> zero(n3, 0.0f);
          for (int q = 0; q < 4; ++q) wr.add_var_f(oname[q], {dk, dj, di}, zero.data(), n3);
          if (!wr.write(out, &err)) die(err);
        }
        const std::string in = indir + pk.dir + iprefix + fname;
        nc3::Reader r;
        if (!r.open(in, &err)) die(err);
        std::vector<float> v[4];
        for (int q = 0; q < 4; ++q) {
          if (!r.read_slab(iname[q], st, ct, sd, &v[q], &err)) die(in + ": " + err);
          if (v[q].size() != np) die(in + ": block size mismatch");
        }
        // kernel order of the files: phase a, amplitude a, phase b, amplitude b
        check(fwant_sgtker_convert(K, conv, v[0].data(), v[1].data(), v[2].data(), v[3].data()), K, "convert");
        for (int q = 0; q < 4; ++q)
          if (!nc3::update_slab(out, oname[q], st, ct, sd, v[q].data(), &err)) die(err);
        ++done;
      }
  }
  return done;
}

}  // namespace

// --info: the kernel statistics of SI_ker2info (code/srcF.kernel/SI_ker2info.F90).
// TomoKernel.conf gives MAIN_CONF and snap_id (init_kernel :422-433); standard input the
// station list, the output directory, the thresholds kap0 kaq0 kbp0 kbq0 and the rank id,
// each read list-directed (:116-129).  Every pick's kernel file
// <pick directory>/kernel_NNN_mpi000000_n00000.nc is read over the snapshot's whole I J K
// (:268-274) and folded in on the device (fwant_kerinfo); the result is
// <output directory>/kerinfo_NNN_mpi000000_n00000.nc (kernelinfo_skel :435-483).
int run_info(const std::string& ker_conf, int device) {
  conf::File kc;
  std::string err;
  if (!kc.load(ker_conf, &err)) die(err);
  std::string main_conf, kid_s;
  if (!kc.get("MAIN_CONF", 2, &main_conf) || !kc.get("snap_id", 2, &kid_s))
    die(ker_conf + ": keys MAIN_CONF and snap_id needed");
  const int kid = to_i(kid_s, "snap_id");
  conf::File cf;
  if (!cf.load(main_conf, &err)) die(err);
  std::vector<seisfd::SnapDef> snaps;
  try {
    const int ni = seisfd::need_int(cf, "ni", 2), nj = seisfd::need_int(cf, "nj", 2), nk = seisfd::need_int(cf, "nk", 2);
    if (cf.has("dims"))
      for (int d = 0; d < 3; ++d)
        if (seisfd::need_int(cf, "dims", d + 2) != 1) die("dims must be 1 1 1: one GPU holds the whole grid");
    snaps = seisfd::read_snaps(cf, ni, nj, nk);
  } catch (const std::exception& e) {
    die(main_conf + ": " + e.what());
  }
  // list-directed records of standard input: a character value is the record's first item
  // (quotes removed), numbers may continue over further records; blank records hold none
  std::string line;
  auto first_item = [&](const char* what) {
    while (std::getline(std::cin, line)) {
      const auto w = words(line);
      if (!w.empty()) return unquote(w[0]);
    }
    die(std::string("standard input: ") + what + " missing");
  };
  auto numbers = [&](size_t n, const char* what) {
    std::vector<std::string> w;
    while (w.size() < n && std::getline(std::cin, line))
      for (const std::string& t : words(line)) w.push_back(t);
    if (w.size() < n) die(std::string("standard input: ") + what + " missing");
    w.resize(n);
    return w;
  };
  const std::string sgt_list = first_item("station list file name");
  const std::string pnm_info = first_item("output directory");
  float k0[4];
  {
    const auto w = numbers(4, "thresholds kap0 kaq0 kbp0 kbq0");
    for (int q = 0; q < 4; ++q) k0[q] = to_f(w[size_t(q)], "threshold");
  }
  std::printf(" input mpi id:\n");
  for (const std::string& t : numbers(3, "rank id (n_i n_j n_k)"))
    if (to_i(t, "rank id") != 0) die("rank id must be 0 0 0: one rank holds the whole grid");

  const seisfd::SnapDef* sp = nullptr;
  for (const seisfd::SnapDef& q : snaps)
    if (q.id == kid) sp = &q;
  if (!sp) die(main_conf + ": snap_" + seisfd::pad(kid, 3) + " missing");
  if (!sp->sgt) {  // kernode_if (:147)
    std::printf("fwant_ker: snapshot series %d holds no stresses: nothing to do\n", kid);
    return 0;
  }
  const int I = sp->subc[0], J = sp->subc[1], Kd = sp->subc[2];
  const size_t np = size_t(I) * J * Kd;
  std::ifstream sl(sgt_list);
  if (!sl) die("sgt_list open err:" + sgt_list);
  fwant_kerinfo* info = nullptr;
  if (fwant_kerinfo_create((long long)np, k0, device, &info) != FWANT_OK)
    die(std::string("kerinfo_create: ") + (info ? fwant_kerinfo_last_error(info) : "error"));
  auto kcheck = [&](fwant_status rc, const char* what) {
    if (rc != FWANT_OK) die(std::string(what) + ": " + fwant_kerinfo_last_error(info));
  };
  // names of the record variables (MAXKSTNM 8, MAXKEVNM 20, :34): a longer or empty name is
  // not stored (the library refuses the write, the reference ignores the error)
  std::vector<std::string> sta_names, evt_names;
  auto tag = [](std::vector<std::string>& names, const std::string& n, size_t maxlen) {
    if (n.empty() || n.size() > maxlen) return 0;
    names.push_back(n);
    return int(names.size());
  };
  static const char* const vname[4] = {"phase_Vp", "amplitude_Vp", "phase_Vs", "amplitude_Vs"};
  const std::string kfile = "/kernel_" + seisfd::pad(kid, 3) + "_" + seisfd::MPI_SUFFIX + "_n00000.nc";
  const std::vector<uint64_t> st0 = {0, 0, 0}, ct = {uint64_t(Kd), uint64_t(J), uint64_t(I)}, sd1 = {1, 1, 1};
  std::vector<float> vol[4];
  long long picks = 0, nevents = 0;
  while (std::getline(sl, line)) {  // sta_loop (:162-340)
    const auto w = words(line);
    if (w.empty() || w[0][0] == '#') continue;
    // KSTNM up to the first blank, the event list next; a single item is the event list
    const std::string sta = w.size() >= 2 ? w[0] : std::string();
    const std::string evt_list = w.size() >= 2 ? w[1] : w[0];
    const std::vector<Event> events = read_events(evt_list, 0, false);
    const int sta_tag = tag(sta_names, sta, 8);
    for (const Event& e : events) {
      bool any = false;
      for (int c = 0; c < 6; ++c) any = any || e.picknum[c] > 0;
      if (!any) continue;  // (:225)
      const int evt_tag = tag(evt_names, e.name, 20);
      for (int c = 0; c < 6; ++c)
        for (const Pick& pk : e.picks[c]) {
          const std::string path = pk.dir + kfile;
          nc3::Reader rd;
          if (!rd.open(path, &err)) die("nfseis_varget: " + err);
          for (int q = 0; q < 4; ++q)
            if (!rd.read_slab(vname[q], st0, ct, sd1, &vol[q], &err)) die(path + ": " + err);
          const float* kp[4] = {vol[0].data(), vol[1].data(), vol[2].data(), vol[3].data()};
          kcheck(fwant_kerinfo_add_pick(info, kp), "add_pick");
          ++picks;
        }
      kcheck(fwant_kerinfo_end_event(info, sta_tag, evt_tag), "end_event");
      ++nevents;
    }
  }
  int nrec = 0;
  kcheck(fwant_kerinfo_records(info, &nrec), "records");
  std::vector<float> S(4 * np);
  std::vector<int> N(4 * np);
  kcheck(fwant_kerinfo_totals(info, S.data(), N.data()), "totals");
  std::vector<int> M[4], rm(4 * np), rs(4 * np), re(4 * np);
  std::vector<char> CS[4], CE[4];
  for (int q = 0; q < 4; ++q) {
    M[q].reserve(size_t(nrec) * np);
    CS[q].assign(size_t(nrec) * np * 8, 0);
    CE[q].assign(size_t(nrec) * np * 20, 0);
  }
  for (int r = 0; r < nrec; ++r) {
    kcheck(fwant_kerinfo_record(info, r, rm.data(), rs.data(), re.data()), "record");
    for (int q = 0; q < 4; ++q) {
      M[q].insert(M[q].end(), rm.begin() + q * np, rm.begin() + (q + 1) * np);
      for (size_t p = 0; p < np; ++p) {
        const int a = rs[q * np + p], b = re[q * np + p];
        if (a > 0) std::memcpy(&CS[q][(size_t(r) * np + p) * 8], sta_names[size_t(a - 1)].data(), sta_names[size_t(a - 1)].size());
        if (b > 0) std::memcpy(&CE[q][(size_t(r) * np + p) * 20], evt_names[size_t(b - 1)].data(), evt_names[size_t(b - 1)].size());
      }
    }
  }
  fwant_kerinfo_destroy(info);
  nc3::Writer wr;
  const int di = wr.add_dim("I", uint64_t(I)), dj = wr.add_dim("J", uint64_t(J)), dk = wr.add_dim("K", uint64_t(Kd));
  const int ds = wr.add_dim("maxkstnm", 8), de = wr.add_dim("maxkevnm", 20), dn = wr.add_dim("N", 0);
  static const char* const sfx[4] = {"ap", "aq", "bp", "bq"};
  static const char* const thn[4] = {"threshold_Kap", "threshold_Kaq", "threshold_Kbp", "threshold_Kbq"};
  for (int q = 0; q < 4; ++q) wr.add_gatt(thn[q], nc3::NC_FLOAT, {double(k0[q])});
  for (int q = 0; q < 4; ++q) wr.add_var_f(std::string("S") + sfx[q], {dk, dj, di}, S.data() + q * np, np);
  for (int q = 0; q < 4; ++q) wr.add_var_i(std::string("N") + sfx[q], {dk, dj, di}, N.data() + q * np, np);
  for (int q = 0; q < 4; ++q) wr.add_var_i(std::string("M") + sfx[q], {dn, dk, dj, di}, M[q].data(), M[q].size());
  for (int q = 0; q < 4; ++q)
    wr.add_var_c(std::string("KSTNM") + sfx[q], {dn, dk, dj, di, ds}, CS[q].data(), CS[q].size());
  for (int q = 0; q < 4; ++q)
    wr.add_var_c(std::string("KEVNM") + sfx[q], {dn, dk, dj, di, de}, CE[q].data(), CE[q].size());
  wr.set_numrecs(uint64_t(nrec));
  const std::string out = pnm_info + "/kerinfo_" + seisfd::pad(kid, 3) + "_" + seisfd::MPI_SUFFIX + "_n00000.nc";
  if (!wr.write(out, &err)) die(err);
  std::printf("fwant_ker: %lld picks of %lld events, %d records into %s\n", picks, nevents, nrec, out.c_str());
  return 0;
}

// --pair: SI_ker_pair (code/srcF.kernel/SI_ker_pair.F90), the kernels of one source-receiver
// pair.  TomoKernel.conf (init_kernel :542-602): MAIN_CONF, SGT_ROOT (the receiver's sgt_
// series), SGT_M0, WAVE_ROOT (the source's sgt_ series), snap_id, block_size, fnm_syn (the
// synthetic: knt, then T V U per line, init_synthetic :633-645), number_of_freqband,
// number_of_measured and the <time_window> list (per measurement a line "band filter t1
// t2", filter 1 one-pass, 2 forward-backward, 3 none, and a line with the output
// directory), then the <filter_file> list.  Standard input: the rank id.  Per block the
// strains of both series, the single-precision scatter (sgt2scatter :738-780) and per band,
// filter and window the kernels (:322-357) into <directory>/kernel_NNN_mpi000000_n00000.nc
// (kernel_phase_Vp kernel_amplitude_Vp kernel_phase_Vs kernel_amplitude_Vs over the
// snapshot's I J K).  The debug exports of export_info (kernel.para.log and the filtered
// synthetics) are not written.
int run_pair(const std::string& ker_conf, int device) {
  conf::File kc;
  std::string err;
  if (!kc.load(ker_conf, &err)) die(err);
  auto kget = [&](const std::string& key, int col) {
    std::string v;
    if (!kc.get(key, col, &v)) die(ker_conf + ": key " + key + " column " + std::to_string(col) + " missing");
    return v;
  };
  const std::string main_conf = kget("MAIN_CONF", 2), pnm_sgt = kget("SGT_ROOT", 2), pnm_wave = kget("WAVE_ROOT", 2);
  const float sgt_m0 = to_f(kget("SGT_M0", 2), "SGT_M0");
  const int kid = to_i(kget("snap_id", 2), "snap_id");
  int blksiz[3];
  for (int d = 0; d < 3; ++d) {
    blksiz[d] = to_i(kget("block_size", d + 2), "block_size");
    if (blksiz[d] == 0 || blksiz[d] < -1) die(ker_conf + ": block_size must be -1 or >= 1");
  }
  const std::string fnm_syn = kget("fnm_syn", 2);
  const int num_freq = to_i(kget("number_of_freqband", 2), "number_of_freqband");
  const int num_meas = to_i(kget("number_of_measured", 2), "number_of_measured");
  // <time_window>: num_meas pairs of lines
  struct Window {
    int freq, filt;  // filt 1 P1, 2 P2, 3 none
    float t1, t2;
    std::string dir;
    int nt1 = 0, nt2 = 0;
  };
  std::vector<Window> wins;
  {
    std::ifstream in(ker_conf);
    std::string line;
    bool found = false;
    while (std::getline(in, line)) {
      const auto w = words(line.substr(0, line.find('#')));
      if (!w.empty() && w[0] == "<time_window>") { found = true; break; }
    }
    if (!found) die(ker_conf + ": <time_window> missing");
    for (int q = 0; q < num_meas; ++q) {
      std::vector<std::string> w;
      while (w.empty()) {
        if (!std::getline(in, line)) die(ker_conf + ": fewer time windows than number_of_measured");
        w = words(line);
      }
      if (w.size() < 4) die(ker_conf + ": a time window needs band, filter, t1 and t2: " + line);
      Window win;
      win.freq = to_i(w[0], "band");
      win.filt = to_i(w[1], "filter");
      win.t1 = to_f(w[2], "t1");
      win.t2 = to_f(w[3], "t2");
      if (win.freq < 1 || win.freq > num_freq || win.filt < 1 || win.filt > 3)
        die(ker_conf + ": band outside 1..number_of_freqband or filter outside 1..3: " + line);
      if (!std::getline(in, line)) die(ker_conf + ": output directory of a time window missing");
      win.dir = trim(line);
      wins.push_back(win);
    }
  }
  const std::vector<Filter> filters = read_filters(ker_conf, num_freq);
  // the synthetic
  std::vector<float> T, V, U;
  int knt = 0;
  {
    std::ifstream f(fnm_syn);
    if (!f) die("cannot open synthetic " + fnm_syn);
    std::string line;
    std::vector<std::string> w;
    while (w.empty() && std::getline(f, line)) w = words(line);
    if (w.empty()) die(fnm_syn + ": knt missing");
    knt = to_i(w[0], fnm_syn);
    if (knt < 2) die(fnm_syn + ": knt must be >= 2");
    std::vector<std::string> vals;
    while (int(vals.size()) < 3 * knt && std::getline(f, line))
      for (const std::string& t : words(line)) vals.push_back(t);
    if (int(vals.size()) < 3 * knt) die(fnm_syn + ": fewer than knt lines of T V U");
    for (int n = 0; n < knt; ++n) {
      T.push_back(to_f(vals[size_t(3 * n)], fnm_syn));
      V.push_back(to_f(vals[size_t(3 * n + 1)], fnm_syn));
      U.push_back(to_f(vals[size_t(3 * n + 2)], fnm_syn));
    }
  }
  // twinlim2num (:647-665): the last T <= t1 and the first T >= t2
  for (Window& w : wins) {
    for (int n = 1; n <= knt; ++n)
      if (T[size_t(n - 1)] <= w.t1 && (w.nt1 == 0 || T[size_t(n - 1)] > T[size_t(w.nt1 - 1)])) w.nt1 = n;
    for (int n = 1; n <= knt; ++n)
      if (T[size_t(n - 1)] >= w.t2 && (w.nt2 == 0 || T[size_t(n - 1)] < T[size_t(w.nt2 - 1)])) w.nt2 = n;
    if (w.nt1 == 0 || w.nt2 == 0 || w.nt1 > w.nt2)
      die(w.dir + ": time window outside the synthetic's time axis");
    const Filter& F = filters[size_t(w.freq - 1)];
    if (w.filt != 3 && F.nod1 < 1) die(w.dir + ": band without filter coefficients");
  }
  conf::File cf;
  if (!cf.load(main_conf, &err)) die(err);
  std::vector<seisfd::SnapDef> snaps;
  double stept_d = 0.0;
  std::string media_root;
  try {
    const int ni = seisfd::need_int(cf, "ni", 2), nj = seisfd::need_int(cf, "nj", 2), nk = seisfd::need_int(cf, "nk", 2);
    if (cf.has("dims"))
      for (int d = 0; d < 3; ++d)
        if (seisfd::need_int(cf, "dims", d + 2) != 1) die("dims must be 1 1 1: one GPU holds the whole grid");
    if (!cf.get_double("stept", 2, &stept_d)) throw std::runtime_error("key stept missing");
    if (!cf.get("MEDIA_ROOT", 2, &media_root)) throw std::runtime_error("key MEDIA_ROOT missing");
    snaps = seisfd::read_snaps(cf, ni, nj, nk);
  } catch (const std::exception& e) {
    die(main_conf + ": " + e.what());
  }
  std::printf(" input mpi id:\n");
  {
    std::vector<std::string> w;
    std::string line;
    while (w.size() < 3 && std::getline(std::cin, line))
      for (const std::string& t : words(line)) w.push_back(t);
    if (w.size() < 3) die("standard input: rank id (n_i n_j n_k) missing");
    for (int d = 0; d < 3; ++d)
      if (to_i(w[size_t(d)], "rank id") != 0) die("rank id must be 0 0 0: one rank holds the whole grid");
  }
  const seisfd::SnapDef* sp = nullptr;
  for (const seisfd::SnapDef& q : snaps)
    if (q.id == kid) sp = &q;
  if (!sp) die(main_conf + ": snap_" + seisfd::pad(kid, 3) + " missing");
  if (!sp->sgt) {  // kernode_if (:172)
    std::printf("fwant_ker: snapshot series %d holds no stresses: nothing to do\n", kid);
    return 0;
  }
  const float kdt = float(sp->tinv) * float(stept_d);
  if (std::fabs((T[1] - T[0]) - kdt) > 1e-6f)
    std::printf("fwant_ker: synthetic time step %g differs from the snapshot's %g\n", double(T[1] - T[0]), double(kdt));
  static const char* const kname[4] = {"kernel_phase_Vp", "kernel_amplitude_Vp", "kernel_phase_Vs",
                                       "kernel_amplitude_Vs"};
  const std::string kfile = "/kernel_" + seisfd::pad(kid, 3) + "_" + seisfd::MPI_SUFFIX + "_n00000.nc";
  {  // nfseis_grid3d_def of every measured window's file (:183-198)
    const size_t n3 = size_t(sp->subc[0]) * sp->subc[1] * sp->subc[2];
    const std::vector<float> zero(n3, 0.0f);
    for (const Window& w : wins) {
      nc3::Writer wr;
      const int di = wr.add_dim("I", uint64_t(sp->subc[0])), dj = wr.add_dim("J", uint64_t(sp->subc[1])),
                dk = wr.add_dim("K", uint64_t(sp->subc[2]));
      wr.add_gatt_text("title", "Finite frequency kernel");
      for (int q = 0; q < 4; ++q) wr.add_var_f(kname[q], {dk, dj, di}, zero.data(), n3);
      if (!wr.write(w.dir + kfile, &err)) die(err);
    }
  }
  int bsz[3], blknum[3];
  for (int d = 0; d < 3; ++d) {
    bsz[d] = blksiz[d] == -1 ? sp->subc[d] : std::min(blksiz[d], sp->subc[d]);
    blknum[d] = (sp->subc[d] + bsz[d] - 1) / bsz[d];
  }
  const std::string media_path = media_root + "/media_" + seisfd::MPI_SUFFIX + ".nc";
  nc3::Reader media;
  if (!media.open(media_path, &err)) die(err);
  fwant_sgtker* K = nullptr;
  size_t k_npts = 0;
  std::vector<float> lam, mu, stress, out[4];
  long long written = 0;
  for (int bk = 1; bk <= blknum[2]; ++bk)
    for (int bj = 1; bj <= blknum[1]; ++bj)
      for (int bi = 1; bi <= blknum[0]; ++bi) {
        const int blk[3] = {bi, bj, bk};
        Geometry g;
        for (int d = 0; d < 3; ++d) {
          g.bsubs[d] = (blk[d] - 1) * bsz[d] + 1;
          g.bsubc[d] = std::min(bsz[d], sp->subc[d] - g.bsubs[d] + 1);
          g.bsubt[d] = 1;
          g.subs[d] = sp->subs[d] + (g.bsubs[d] - 1) * sp->subt[d];
          g.subt[d] = sp->subt[d];
        }
        const size_t np = g.npts();
        if (!K || k_npts != np) {
          if (K) fwant_sgtker_destroy(K);
          K = nullptr;
          check(fwant_sgtker_create((long long)np, knt, double(kdt), device, &K), nullptr, "sgtker_create");
          k_npts = np;
        }
        const std::vector<uint64_t> st = {uint64_t(g.subs[2] - 1), uint64_t(g.subs[1] - 1), uint64_t(g.subs[0] - 1)};
        const std::vector<uint64_t> ct = {uint64_t(g.bsubc[2]), uint64_t(g.bsubc[1]), uint64_t(g.bsubc[0])};
        const std::vector<uint64_t> sd = {uint64_t(g.subt[2]), uint64_t(g.subt[1]), uint64_t(g.subt[0])};
        if (!media.read_slab("lambda", st, ct, sd, &lam, &err) || !media.read_slab("mu", st, ct, sd, &mu, &err))
          die(media_path + ": " + err);
        check(fwant_sgtker_set_media(K, lam.data(), mu.data()), K, "media");
        read_sgt(pnm_sgt, *sp, g, knt, stress);  // the receiver (SGT_ROOT)
        check(fwant_sgtker_set_sgt(K, 0, stress.data()), K, "receiver SGT");
        read_sgt(pnm_wave, *sp, g, knt, stress);  // the source (WAVE_ROOT)
        check(fwant_sgtker_set_sgt(K, 3, stress.data()), K, "source SGT");
        check(fwant_sgtker_scatter_pair(K), K, "scatter_pair");
        for (auto& o : out) o.assign(np, 0.0f);
        const std::vector<uint64_t> kst = {uint64_t(g.bsubs[2] - 1), uint64_t(g.bsubs[1] - 1), uint64_t(g.bsubs[0] - 1)};
        const std::vector<uint64_t> kct = {uint64_t(g.bsubc[2]), uint64_t(g.bsubc[1]), uint64_t(g.bsubc[0])};
        const std::vector<uint64_t> ksd = {1, 1, 1};
        // bands, filter types P1 P2 none, windows in the reference's order (:322-357)
        for (int nfq = 1; nfq <= num_freq; ++nfq)
          for (int npt = 1; npt <= 3; ++npt)
            for (const Window& w : wins) {
              if (w.freq != nfq || w.filt != npt) continue;
              const Filter& F = filters[size_t(nfq - 1)];
              const int mode = npt == 3 ? 0 : npt;
              check(fwant_sgtker_kernel_pair(K, V.data(), U.data(), w.nt1, w.nt2, sgt_m0, mode,
                                             mode ? F.nod1 : 0, mode ? F.b.data() : nullptr,
                                             mode ? F.a.data() : nullptr, out[0].data(), out[1].data(),
                                             out[2].data(), out[3].data()),
                    K, "kernel_pair");
              for (int q = 0; q < 4; ++q)
                if (!nc3::update_slab(w.dir + kfile, kname[q], kst, kct, ksd, out[q].data(), &err)) die(err);
              ++written;
            }
      }
  if (K) fwant_sgtker_destroy(K);
  std::printf("fwant_ker: %lld pair kernel blocks written\n", written);
  return 0;
}

int main(int argc, char** argv) {
  if (argc >= 2 && std::strncmp(argv[1], "--nc-", 5) == 0) return nc_tool(argc, argv);
  std::string ker_conf;
  int device = 0;
  bool lamu = false;  // --lamu: the lambda/mu kernels of SI_ker_sta_lamu
  int conv = 0;       // --convert: 1 lamu2kamu, 2 lamu2vpvs, 3 vpvs2kamu
  bool eq = false;    // --eq: SI_ker_EQ's time shift of the Z-force SGT
  bool info = false;  // --info: the kernel statistics of SI_ker2info
  bool pair = false;  // --pair: SI_ker_pair, one source-receiver pair
  for (int a = 1; a < argc; ++a) {
    const std::string s = argv[a];
    if (s == "--device" && a + 1 < argc) device = std::atoi(argv[++a]);
    else if (s == "--lamu") lamu = true;
    else if (s == "--info") info = true;
    else if (s == "--pair") pair = true;
    else if (s == "--eq") eq = true;
    else if (s == "--convert" && a + 1 < argc) {
      const std::string m = argv[++a];
      conv = m == "lamu2kamu" ? 1 : (m == "lamu2vpvs" ? 2 : (m == "vpvs2kamu" ? 3 : 0));
      if (!conv) die("--convert: mode must be lamu2kamu, lamu2vpvs or vpvs2kamu");
    } else ker_conf = s;
  }
  if (conv && (lamu || eq)) die("--convert excludes --lamu and --eq");
  if (info && (conv || lamu || eq)) die("--info excludes --convert, --lamu and --eq");
  if (pair && (conv || lamu || eq || info)) die("--pair excludes --convert, --lamu, --eq and --info");
  if (ker_conf.empty()) ker_conf = conv ? "TomoKernel_conv.conf" : "TomoKernel.conf";
  if (info) return run_info(ker_conf, device);
  if (pair) return run_pair(ker_conf, device);
  // init_kernel (SI_ker_sta.F90:1047-1082)
  conf::File kc;
  std::string err;
  if (!kc.load(ker_conf, &err)) die(err);
  auto kget = [&](const std::string& key, int col) {
    std::string v;
    if (!kc.get(key, col, &v)) die(ker_conf + ": key " + key + " column " + std::to_string(col) + " missing");
    return v;
  };
  const std::string main_conf = kget("MAIN_CONF", 2);
  const int kid = to_i(kget("snap_id", 2), "snap_id");
  const bool first_run = parse_logical(kget("first_run", 2), "first_run");
  int bstart[3], bcount[3], bstride[3], blkfst[3], blksiz[3];
  for (int d = 0; d < 3; ++d) {
    bstart[d] = to_i(kget("sub_start", d + 2), "sub_start");
    bcount[d] = to_i(kget("sub_count", d + 2), "sub_count");
    bstride[d] = to_i(kget("sub_stride", d + 2), "sub_stride");
    blkfst[d] = to_i(kget("block_from", d + 2), "block_from");
    blksiz[d] = to_i(kget("block_size", d + 2), "block_size");
    if (bstart[d] < 1 || bstride[d] < 1 || blkfst[d] < 1 || blksiz[d] == 0 || blksiz[d] < -1)
      die(ker_conf + ": sub_start, sub_stride, block_from >= 1 and block_size -1 or >= 1");
  }
  const int knt = to_i(kget("SGT_TIMEDIM_SIZE", 2), "SGT_TIMEDIM_SIZE");
  const float sgt_m0 = to_f(kget("SGT_M0", 2), "SGT_M0");
  const std::string sgt_root = kget("SGT_ROOT", 2), event_root = kget("EVENT_ROOT", 2),
                    event_outd = kget("EVENT_OUTD", 2);
  const std::string sgt_sta[3] = {kget("SGT_STAX", 2), kget("SGT_STAY", 2), kget("SGT_STAZ", 2)};
  const int num_freq = to_i(kget("number_of_freqband", 2), "number_of_freqband");
  if (knt < 2) die(ker_conf + ": SGT_TIMEDIM_SIZE must be >= 2");

  // the solver's configuration (para_init, io_snap_read, media_fnm_init)
  conf::File cf;
  if (!cf.load(main_conf, &err)) die(err);
  std::vector<seisfd::SnapDef> snaps;
  int ni, nj, nk;
  double stept_d;
  std::string media_root;
  try {
    ni = seisfd::need_int(cf, "ni", 2);
    nj = seisfd::need_int(cf, "nj", 2);
    nk = seisfd::need_int(cf, "nk", 2);
    if (cf.has("dims"))
      for (int d = 0; d < 3; ++d)
        if (seisfd::need_int(cf, "dims", d + 2) != 1) die("dims must be 1 1 1: one GPU holds the whole grid");
    if (!cf.get_double("stept", 2, &stept_d)) throw std::runtime_error("key stept missing");
    if (!cf.get("MEDIA_ROOT", 2, &media_root)) throw std::runtime_error("key MEDIA_ROOT missing");
    snaps = seisfd::read_snaps(cf, ni, nj, nk);
  } catch (const std::exception& e) {
    die(main_conf + ": " + e.what());
  }
  const std::vector<Filter> filters = read_filters(ker_conf, num_freq);

  // standard input: (conversions: the input directory, one line, may be blank) the station
  // list file, then the rank id (read *, n_i, n_j, n_k)
  std::string sgt_list, line, indir;
  if (conv) {
    if (!std::getline(std::cin, line)) die("standard input: input directory line missing");
    indir = unquote(trim(line));
  }
  while (sgt_list.empty() && std::getline(std::cin, line)) sgt_list = unquote(trim(line));
  if (sgt_list.empty()) die("standard input: station list file name missing");
  {
    std::vector<std::string> w;
    while (w.size() < 3 && std::getline(std::cin, line))
      for (const std::string& t : words(line)) w.push_back(t);
    if (w.size() < 3) die("standard input: rank id (n_i n_j n_k) missing");
    for (int d = 0; d < 3; ++d)
      if (to_i(w[size_t(d)], "rank id") != 0) die("rank id must be 0 0 0: one rank holds the whole grid");
  }

  // the snapshot series of the SGTs (kernode_if: it must hold stresses)
  const seisfd::SnapDef* sp = nullptr;
  for (const seisfd::SnapDef& s : snaps)
    if (s.id == kid) sp = &s;
  if (!sp) die(main_conf + ": snap_" + seisfd::pad(kid, 3) + " missing");
  if (!sp->sgt) {
    std::printf("fwant_ker: snapshot series %d holds no stresses: nothing to do\n", kid);
    return 0;
  }
  // kernel points in the snapshot's sample grid (SI_ker_sta.F90:179-236 for one rank:
  // subnc_s = sub_start, subnc_t = sub_stride, subnc_c the points up to the series' end)
  int subnc_s[3], subnc_c[3], subnc_t[3], bsz[3], blknum[3];
  for (int d = 0; d < 3; ++d) {
    int gc = (sp->subc[d] - bstart[d]) / bstride[d] + 1;
    if (bcount[d] != -1 && bcount[d] < gc) gc = bcount[d];
    if (bstart[d] > sp->subc[d] || gc < 1) die(ker_conf + ": sub_start / sub_count select no snapshot point");
    subnc_s[d] = bstart[d];
    subnc_c[d] = gc;
    subnc_t[d] = bstride[d];
    bsz[d] = (blksiz[d] == -1 || blksiz[d] > gc) ? gc : blksiz[d];
    blknum[d] = (gc + bsz[d] - 1) / bsz[d];
  }
  const float kdt = float(sp->tinv) * float(stept_d);  // kdt = sub_gtinv * stept, single precision
  const float tmin = kdt, tmax = float(knt) * kdt;
  const std::string media_path = media_root + "/media_" + seisfd::MPI_SUFFIX + ".nc";
  nc3::Reader media;
  if (!media.open(media_path, &err)) die(err);

  std::ifstream sl(sgt_list);
  if (!sl) die("sgt_list open err: " + sgt_list);
  fwant_sgtker* K = nullptr;
  size_t k_npts = 0;
  long long written = 0;
  std::vector<float> lam, mu, stress;
  // variable names and file prefix: SI_ker_sta.F90:736-743, SI_ker_sta_lamu.F90:736-743
  static const char* const kname_vpvs[4] = {"phase_Vp", "amplitude_Vp", "phase_Vs", "amplitude_Vs"};
  static const char* const kname_lamu[4] = {"phase_la", "amplitude_la", "phase_mu", "amplitude_mu"};
  static const char* const kname_kamu[4] = {"phase_ka", "amplitude_ka", "phase_mu", "amplitude_mu"};
  const char* const* kname = (lamu || conv == 1 || conv == 2) ? kname_lamu : kname_vpvs;  // kernel run / input
  const std::string kprefix = (lamu || conv == 1 || conv == 2) ? "/kernel_lamu_" : "/kernel_";
  // conversions: output names and file prefix (SI_ker_lamu2kamu.F90:741-748, SI_ker_lamu2vpvs.F90:741-748,
  // SI_ker_vpvs2kamu.F90:741-748)
  const char* const* oname = conv == 3 ? kname_kamu : kname_vpvs;
  const std::string oprefix = conv == 3 ? "/kernel_kamu_" : "/kernel_";
  while (std::getline(sl, line)) {
    const auto w = words(line);
    if (w.empty()) continue;
    const std::string sta = unquote(w[0]);
    if (sta.empty() || sta[0] == '#') continue;
    if (w.size() < 2) die(sgt_list + ": a station line needs a name and an event list: " + line);
    const std::vector<Event> events = read_events(unquote(w[1]), num_freq);
    std::printf("fwant_ker: station %s, %zu events, %d x %d x %d blocks\n", sta.c_str(), events.size(), blknum[0],
                blknum[1], blknum[2]);
    for (int bk = blkfst[2]; bk <= blknum[2]; ++bk)
      for (int bj = blkfst[1]; bj <= blknum[1]; ++bj)
        for (int bi = blkfst[0]; bi <= blknum[0]; ++bi) {
          const int blk[3] = {bi, bj, bk};
          const bool first_block = bi == 1 && bj == 1 && bk == 1;
          Geometry g;
          for (int d = 0; d < 3; ++d) {
            g.bsubs[d] = (blk[d] - 1) * bsz[d] * subnc_t[d] + subnc_s[d];
            g.bsubc[d] = std::min(bsz[d], subnc_c[d] - (g.bsubs[d] - subnc_s[d]) / subnc_t[d]);
            g.bsubt[d] = subnc_t[d];
            g.subs[d] = sp->subs[d] + (g.bsubs[d] - 1) * sp->subt[d];
            g.subt[d] = sp->subt[d] * g.bsubt[d];
          }
          const size_t np = g.npts();
          if (!K || k_npts != np) {
            if (K) fwant_sgtker_destroy(K);
            K = nullptr;
            check(fwant_sgtker_create((long long)np, knt, double(kdt), device, &K), nullptr, "sgtker_create");
            if (lamu) check(fwant_sgtker_set_param(K, 1), K, "sgtker_set_param");
            k_npts = np;
          }
          {  // lambda and mu at the block's points (nfseis_varget with subs/subc/subt)
            const std::vector<uint64_t> st = {uint64_t(g.subs[2] - 1), uint64_t(g.subs[1] - 1), uint64_t(g.subs[0] - 1)};
            const std::vector<uint64_t> ct = {uint64_t(g.bsubc[2]), uint64_t(g.bsubc[1]), uint64_t(g.bsubc[0])};
            const std::vector<uint64_t> sd = {uint64_t(g.subt[2]), uint64_t(g.subt[1]), uint64_t(g.subt[0])};
            if (!media.read_slab("lambda", st, ct, sd, &lam, &err) || !media.read_slab("mu", st, ct, sd, &mu, &err))
              die(media_path + ": " + err);
            check(fwant_sgtker_set_media(K, lam.data(), mu.data()), K, "media");
          }
          if (conv) {  // the conversion programs: kernel files in, converted kernel files out
            written += convert_block(K, conv, events, g, *sp, kid, knt, kdt, tmin, tmax, first_run && first_block,
                                     indir, kprefix, kname, oprefix, oname);
            continue;
          }
          bool have[3] = {false, false, false};  // station SGTs on the device for this block
          for (const Event& e : events) {
            const bool rot_any = e.picknum[3] > 0 || e.picknum[4] > 0 || e.picknum[5] > 0;
            bool ud[3], any = false;
            for (int c = 0; c < 6; ++c) any = any || e.picknum[c] > 0;
            std::vector<float> T(static_cast<size_t>(knt)), V[3], U[3];
            for (int n = 0; n < knt; ++n) T[size_t(n)] = float(n + 1) * kdt;
            for (int c = 0; c < 3; ++c) {
              ud[c] = e.picknum[c] > 0 || rot_any;
              if (ud[c]) read_synthetic(e.syn[c], knt, T, V[c], U[c]);
            }
            if (!any) continue;
            for (int c = 0; c < 3; ++c)
              if (ud[c] && !have[c]) {
                read_sgt(sgt_root + "/" + sta + "/" + sgt_sta[c], *sp, g, knt, stress);
                if (eq && c == 2) shift_frames(stress, knt, g.npts(), EQ_SHIFT);
                check(fwant_sgtker_set_sgt(K, c, stress.data()), K, "station SGT");
                have[c] = true;
              }
            read_sgt(event_root + "/" + e.name + "/" + event_outd, *sp, g, knt, stress);
            check(fwant_sgtker_set_sgt(K, 3, stress.data()), K, "event SGT");
            check(fwant_sgtker_scatter(K, (ud[0] ? 1 : 0) | (ud[1] ? 2 : 0) | (ud[2] ? 4 : 0), 1, knt), K, "scatter");
            for (int ncmp = 1; ncmp <= 6; ++ncmp) {
              if (ncmp == 4 && rot_any) {  // syn_rotate of V and U, scatter_rotate (SI_ker_sta.F90:584-589)
                syn_rotate(V, e.rot);
                syn_rotate(U, e.rot);
                double rd[9];
                for (int q = 0; q < 9; ++q) rd[q] = double(e.rot[q]);
                check(fwant_sgtker_rotate(K, rd), K, "rotate");
              }
              const int comp = (ncmp - 1) % 3;
              for (const Pick& pk : e.picks[ncmp - 1]) {
                int nt1, nt2;
                if (!pick_window(pk, T, tmin, tmax, &nt1, &nt2)) continue;
                const std::string path = pk.dir + kprefix + seisfd::pad(kid, 3) + "_" + seisfd::MPI_SUFFIX + "_n00000.nc";
                if (first_run && first_block) {  // nfseis_grid3d_def over the snapshot's points
                  nc3::Writer wr;
                  const int di = wr.add_dim("I", uint64_t(sp->subc[0])), dj = wr.add_dim("J", uint64_t(sp->subc[1])),
                            dk = wr.add_dim("K", uint64_t(sp->subc[2]));
                  wr.add_gatt_text("title", "Finite frequency kernel");
                  const size_t n3 = size_t(sp->subc[0]) * sp->subc[1] * sp->subc[2];
                  const std::vector<float> zero(n3, 0.0f);
                  for (int q = 0; q < 4; ++q) wr.add_var_f(kname[q], {dk, dj, di}, zero.data(), n3);
                  if (!wr.write(path, &err)) die(err);
                }
                if (pk.freq < 1 || (pk.filt != 0 && filters[size_t(pk.freq - 1)].nod1 == 0))
                  die("pick " + pk.dir + ": frequency band without filter coefficients");
                const Filter* F = pk.filt != 0 ? &filters[size_t(pk.freq - 1)] : nullptr;
                std::vector<double> kout[4];
                for (auto& v : kout) v.assign(np, 0.0);
                check(fwant_sgtker_kernel_filtered(K, comp + 1, V[comp].data(), U[comp].data(), nt1, nt2,
                                                   double(sgt_m0), pk.filt, F ? F->nod1 : 0, F ? F->b.data() : nullptr,
                                                   F ? F->a.data() : nullptr, kout[0].data(), kout[1].data(),
                                                   kout[2].data(), kout[3].data()),
                      K, "kernel");
                const std::vector<uint64_t> st = {uint64_t(g.bsubs[2] - 1), uint64_t(g.bsubs[1] - 1),
                                                  uint64_t(g.bsubs[0] - 1)};
                const std::vector<uint64_t> ct = {uint64_t(g.bsubc[2]), uint64_t(g.bsubc[1]), uint64_t(g.bsubc[0])};
                const std::vector<uint64_t> sd = {uint64_t(g.bsubt[2]), uint64_t(g.bsubt[1]), uint64_t(g.bsubt[0])};
                std::vector<float> f(np);
                for (int q = 0; q < 4; ++q) {
                  for (size_t p = 0; p < np; ++p) f[p] = float(kout[q][p]);
                  if (!nc3::update_slab(path, kname[q], st, ct, sd, f.data(), &err)) die(err);
                }
                ++written;
              }
            }
          }
        }
  }
  if (K) fwant_sgtker_destroy(K);
  std::printf("fwant_ker: %lld kernel blocks %s\n", written, conv ? "converted" : "written");
  return 0;
}
