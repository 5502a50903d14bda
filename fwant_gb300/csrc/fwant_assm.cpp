// fwant_assm: the kernel assembly program over the C ABI, a drop-in for the reference's
// SI_ker2assm (code/srcF.kernel/SI_ker2assm.F90, phase-delay kernels) and, with --kamu,
// SI_ker_kamu2assm (kernel_kamu_ files, phase_ka / phase_mu) or, with --lamu,
// SI_ker_lamu2assm (kernel_lamu_ files, phase_la / phase_mu; SI_ker_lamu2assm.F90:290-297)
// on one rank.
//
// Inputs as the reference reads them: TomoKernel.conf (MAIN_CONF, snap_id: init_kernel
// :437-449) and the main configuration's snapshot snap_id, whose subc is the kernel volume;
// on standard input the station list, the inversion block file, the spool directory, the
// four C factors (Cap0 Caq0 Cbp0 Cbq0) and the four thresholds (kap0 kaq0 kbp0 kbq0)
// (:108-120); the inversion block file's block and max_pix dimensions and volume,
// num_of_pix, indx_of_pix variables (init_inv_block :466-485); the station list's lines
// "station event_list"; the event lists' event lines (name, six pick counts, rotation
// matrix), three synthetic-file lines and pick lines (band, filter, t1, t2, kernel
// directory) (:169-280).  For every pick the kernel file
// <kernel directory>/kernel_NNN_mpi000000_n00000.nc is projected onto the blocks on the
// GPU (fwant_assm_project), the block values are scaled by the C factors and written as
// compact rows (export_G_compact :545-571) to <spool>/<directory with '/' as '_'>.Kap.unformat
// and .Kbp.unformat; at the end inv_G_band.conf (export_inv_info :573-585) and the scaled
// sums inv_G_sum.Kap.unformat / .Kbp.unformat (export_G_sum :587-598).
//
// Usage: fwant_assm [TomoKernel.conf] [--kamu | --lamu] [--device N] < answers
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "conf.h"
#include "fwant_assm.h"
#include "netcdf3.h"
#include "seisfd_conf.h"

namespace {

[[noreturn]] void die(const std::string& m) {
  std::fprintf(stderr, "fwant_assm: %s\n", m.c_str());
  std::exit(1);
}

std::string trim(const std::string& s) {
  const size_t a = s.find_first_not_of(" \t\r\n");
  if (a == std::string::npos) return "";
  return s.substr(a, s.find_last_not_of(" \t\r\n") - a + 1);
}

std::vector<std::string> words(const std::string& s) {
  std::istringstream in(s);
  std::vector<std::string> w;
  for (std::string t; in >> t;) w.push_back(t);
  return w;
}

int to_i(const std::string& s, const std::string& where) {
  char* end = nullptr;
  const long v = std::strtol(s.c_str(), &end, 10);
  if (end == s.c_str() || *end != '\0') throw std::runtime_error(where + ": not an integer: " + s);
  return int(v);
}

// Fortran unformatted sequential record: 4-byte length, payload, 4-byte length
void record(std::ofstream& f, const void* p, uint32_t n) {
  f.write(reinterpret_cast<const char*>(&n), 4);
  if (n) f.write(static_cast<const char*>(p), n);
  f.write(reinterpret_cast<const char*>(&n), 4);
}

// splash2underline (:529-543): drop the leading '.' and '/' characters, then '/' -> '_'
std::string splash2underline(const std::string& pnm) {
  std::string s = pnm;
  size_t q = 0;
  while (q < s.size() && (s[q] == '.' || s[q] == '/')) ++q;
  s = trim(s.substr(q));
  for (char& c : s)
    if (c == '/') c = '_';
  return s;
}

// export_G_compact: the blocks with |B| > ker0, as (num_blk, ker0), (ncoef), (index, value)*
int export_compact(const std::vector<float>& B, float ker0, const std::string& path) {
  std::vector<unsigned char> pairs;
  int ncoef = 0;
  for (size_t n = 0; n < B.size(); ++n)
    if (std::fabs(B[n]) > ker0) {
      const int32_t idx = int32_t(n + 1);
      const float v = B[n];
      const auto* pi = reinterpret_cast<const unsigned char*>(&idx);
      const auto* pv = reinterpret_cast<const unsigned char*>(&v);
      pairs.insert(pairs.end(), pi, pi + 4);
      pairs.insert(pairs.end(), pv, pv + 4);
      ++ncoef;
    }
  std::ofstream f(path, std::ios::binary | std::ios::trunc);
  if (!f) die("cannot write " + path);
  unsigned char head[8];
  const int32_t nb = int32_t(B.size());
  std::copy_n(reinterpret_cast<const unsigned char*>(&nb), 4, head);
  std::copy_n(reinterpret_cast<const unsigned char*>(&ker0), 4, head + 4);
  record(f, head, 8);
  const int32_t nc = ncoef;
  record(f, &nc, 4);
  record(f, pairs.data(), uint32_t(pairs.size()));
  if (!f) die("write error on " + path);
  return ncoef;
}

// export_G_sum: (num_blk), (values)
void export_sum(const std::vector<float>& S, const std::string& path) {
  std::ofstream f(path, std::ios::binary | std::ios::trunc);
  if (!f) die("cannot write " + path);
  const int32_t nb = int32_t(S.size());
  record(f, &nb, 4);
  record(f, S.data(), uint32_t(S.size() * sizeof(float)));
  if (!f) die("write error on " + path);
}

// the next line of standard input ("(a)" reads)
std::string stdin_line(const char* what) {
  std::string l;
  if (!std::getline(std::cin, l)) die(std::string("standard input: ") + what + " missing");
  return trim(l);
}

// n list-directed real(SP) values from standard input (a record may take several lines)
std::vector<float> stdin_reals(size_t n, const char* what) {
  std::vector<float> v;
  std::string l;
  while (v.size() < n) {
    if (!std::getline(std::cin, l)) die(std::string("standard input: ") + what + " missing");
    for (char& c : l)
      if (c == ',') c = ' ';
    for (const std::string& t : words(l)) {
      if (v.size() == n) break;
      v.push_back(conf::to_float(t, "standard input"));
    }
  }
  return v;
}

struct Blocks {
  int num_blk = 0, max_pix = 0;
  std::vector<float> volume;  // (max_pix, num_blk)
  std::vector<int> npix;      // (num_blk)
  std::vector<int> pixs;      // (3, max_pix, num_blk)
};

Blocks read_blocks(const std::string& path) {
  nc3::Reader r;
  std::string err;
  if (!r.open(path, &err)) die(err);
  const nc3::Dim* db = r.dim("block");
  const nc3::Dim* dp = r.dim("max_pix");
  if (!db || !dp) die(path + ": dimensions block and max_pix required");
  Blocks b;
  b.num_blk = int(db->len);
  b.max_pix = int(dp->len);
  if (!r.read("volume", &b.volume, &err) || !r.read("num_of_pix", &b.npix, &err) ||
      !r.read("indx_of_pix", &b.pixs, &err))
    die(path + ": " + err);
  const size_t np = size_t(b.num_blk) * b.max_pix;
  if (b.volume.size() != np || b.npix.size() != size_t(b.num_blk) || b.pixs.size() != 3 * np)
    die(path + ": variable sizes do not match block x max_pix");
  return b;
}

struct Pick {
  std::string dir;
};

// one event list: the pick lines of every event with picks (:212-280)
std::vector<Pick> read_picks(const std::string& path) {
  std::ifstream in(path);
  if (!in) die("evt_list open err:" + path);
  std::vector<Pick> out;
  std::string line;
  while (std::getline(in, line)) {
    const std::string t = trim(line);
    if (t.empty() || t[0] == '#') continue;
    const auto w = words(t);
    if (w.size() < 16) die(path + ": event line needs a name, 6 pick counts and 9 matrix entries: " + t);
    int picknum[6], total = 0;
    for (int c = 0; c < 6; ++c) {
      picknum[c] = to_i(w[1 + c], path);
      total += picknum[c] > 0 ? picknum[c] : 0;
    }
    for (int c = 0; c < 3; ++c)
      if (!std::getline(in, line)) die(path + ": synthetic file name missing");
    for (int p = 0; p < total; ++p) {
      std::string pl;
      do {
        if (!std::getline(in, line)) die("read event pick error");
        pl = trim(line);
      } while (!pl.empty() && pl[0] == '#');
      // band, filter, t1, t2, then the rest of the line is the kernel directory
      size_t pos = 0;
      for (int k = 0; k < 4; ++k) {
        pos = pl.find_first_not_of(" \t", pos);
        if (pos == std::string::npos) die(path + ": pick line needs band, filter, t1, t2 and a directory: " + pl);
        pos = pl.find_first_of(" \t", pos);
        if (pos == std::string::npos) die(path + ": pick line needs band, filter, t1, t2 and a directory: " + pl);
      }
      Pick pk;
      pk.dir = trim(pl.substr(pos));
      if (pk.dir.empty()) die(path + ": pick line without a kernel directory: " + pl);
      out.push_back(pk);
    }
  }
  return out;
}

int run(int argc, char** argv) {
  std::string ker_conf = "TomoKernel.conf";
  int device = 0;
  bool kamu = false, lamu = false;
  for (int a = 1; a < argc; ++a) {
    const std::string s = argv[a];
    if (s == "--device" && a + 1 < argc) device = std::atoi(argv[++a]);
    else if (s == "--kamu") kamu = true;
    else if (s == "--lamu") lamu = true;
    else ker_conf = s;
  }
  if (kamu && lamu) die("--kamu and --lamu exclude each other");
  const conf::Text kc(ker_conf);
  const std::string main_conf = kc.get("MAIN_CONF", 2);
  const int kid = kc.get_int("snap_id", 2);
  conf::File cf;
  std::string err;
  if (!cf.load(main_conf, &err)) die(err);
  const int ni = seisfd::need_int(cf, "ni", 2), nj = seisfd::need_int(cf, "nj", 2), nk = seisfd::need_int(cf, "nk", 2);
  if (cf.has("dims"))
    for (int d = 0; d < 3; ++d)
      if (seisfd::need_int(cf, "dims", d + 2) != 1) die("dims must be 1 1 1: one rank holds the whole kernel");
  const seisfd::SnapDef* sp = nullptr;
  const std::vector<seisfd::SnapDef> snaps = seisfd::read_snaps(cf, ni, nj, nk);
  for (const auto& s : snaps)
    if (s.id == kid) sp = &s;
  if (!sp) die(main_conf + ": snap_" + seisfd::pad(kid, 3) + " missing");
  const int ki = sp->subc[0], kj = sp->subc[1], kk = sp->subc[2];
  const size_t nvol = size_t(ki) * kj * kk;

  const std::string sgt_list = stdin_line("station list"), fnm_invblk = stdin_line("inversion block file"),
                    pnm_spool = stdin_line("spool directory");
  const std::vector<float> C = stdin_reals(4, "C factors"), K0 = stdin_reals(4, "thresholds");
  std::printf(" %s\n %s\n %s\n", sgt_list.c_str(), fnm_invblk.c_str(), pnm_spool.c_str());
  const float Cap0 = C[0], Cbp0 = C[2], kap0 = K0[0], kbp0 = K0[2];

  const Blocks blk = read_blocks(fnm_invblk);
  fwant_assm* A = nullptr;
  const fwant_status rc = fwant_assm_create(ki, kj, kk, blk.num_blk, blk.max_pix, blk.volume.data(), blk.npix.data(),
                                            blk.pixs.data(), device, &A);
  if (rc != FWANT_OK) die(std::string("inversion blocks: ") + (A ? fwant_assm_last_error(A) : "create failed"));
  std::printf("assemble phase-delay kernel ...\n");

  const std::string prefix = kamu ? "kernel_kamu_" : (lamu ? "kernel_lamu_" : "kernel_");
  const char* const vname[2] = {kamu ? "phase_ka" : (lamu ? "phase_la" : "phase_Vp"),
                                (kamu || lamu) ? "phase_mu" : "phase_Vs"};
  int max_bdap = 0, max_bdbp = 0;
  double gpu_ms = 0.0;
  long npicks = 0;
  std::vector<float> Ka, Kb, B(size_t(blk.num_blk) * 2);
  std::ifstream sl(sgt_list);
  if (!sl) die("sgt_list open err:" + sgt_list);
  for (std::string line; std::getline(sl, line);) {
    const std::string t = trim(line);
    if (t.empty() || t[0] == '#') continue;
    const auto w = words(t);
    if (w.size() < 2) die(sgt_list + ": a station line needs a name and an event list: " + t);
    for (const Pick& pk : read_picks(w[1])) {
      const std::string path = pk.dir + "/" + prefix + seisfd::pad(kid, 3) + "_" + seisfd::MPI_SUFFIX + "_n00000.nc";
      nc3::Reader r;
      if (!r.open(path, &err) || !r.read(vname[0], &Ka, &err) || !r.read(vname[1], &Kb, &err)) die(err);
      if (Ka.size() != nvol || Kb.size() != nvol) die(path + ": kernel volume is not the snapshot's subc");
      const float* kp[2] = {Ka.data(), Kb.data()};
      if (fwant_assm_project(A, 2, kp, B.data()) != FWANT_OK) die(fwant_assm_last_error(A));
      double ms = 0.0;
      fwant_assm_last_ms(A, &ms);
      gpu_ms += ms;
      ++npicks;
      std::vector<float> Bap(B.begin(), B.begin() + blk.num_blk), Bbp(B.begin() + blk.num_blk, B.end());
      for (float& v : Bap) v = v * Cap0;
      for (float& v : Bbp) v = v * Cbp0;
      const std::string part = pnm_spool + "/" + splash2underline(pk.dir);
      const int cur_bdap = export_compact(Bap, kap0, part + ".Kap.unformat");
      const int cur_bdbp = export_compact(Bbp, kbp0, part + ".Kbp.unformat");
      max_bdap = std::max(max_bdap, cur_bdap);
      max_bdbp = std::max(max_bdbp, cur_bdbp);
      std::printf(" G_band= %d %d %d %d %d\n", cur_bdap, 0, cur_bdbp, 0, std::max(max_bdap, max_bdbp));
    }
  }
  {
    const std::string path = pnm_spool + "/inv_G_band.conf";
    std::FILE* f = std::fopen(path.c_str(), "w");
    if (!f) die("cannot write " + path);
    std::fprintf(f, "max_band_width_Kap = %12d\nmax_band_width_Kaq = %12d\nmax_band_width_Kbp = %12d\n"
                    "max_band_width_Kbq = %12d\n", max_bdap, 0, max_bdbp, 0);
    std::fclose(f);
  }
  std::vector<float> S(size_t(blk.num_blk) * 4);
  if (fwant_assm_sums(A, S.data()) != FWANT_OK) die(fwant_assm_last_error(A));
  std::vector<float> Sap(S.begin(), S.begin() + blk.num_blk), Sbp(S.begin() + blk.num_blk, S.begin() + 2 * blk.num_blk);
  for (float& v : Sap) v = v * Cap0;
  for (float& v : Sbp) v = v * Cbp0;
  export_sum(Sap, pnm_spool + "/inv_G_sum.Kap.unformat");
  export_sum(Sbp, pnm_spool + "/inv_G_sum.Kbp.unformat");
  std::printf("%ld picks assembled onto %d blocks; projection on the GPU: %.3f ms\n", npicks, blk.num_blk, gpu_ms);
  fwant_assm_destroy(A);
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
