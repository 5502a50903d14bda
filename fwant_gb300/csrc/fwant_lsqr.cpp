// fwant_lsqr — the damped and smoothed tomographic inversion (inv.LSQR/solver_damp_smooth.f90
// and, with --loc, solver_damp_smo_loc.f90) with the LSQR iteration on the GPU through the
// C ABI (include/fwant_lsqr.h).
//
// Standard input as the reference reads it (solver_damp_smooth.f90:57-84): mode (1 = simple
// damping), damping and smoothing weights, number of structure components, station terms
// per measurement and their weight, event terms and weight, the data list file, the
// smoothing operator file, the kernel and data thresholds.  With --loc the order of
// solver_damp_smo_loc.f90 (mode, data list, smoothing file, components, station terms,
// event terms, location terms and weight, damping and smoothing, thresholds).
//
// The data list holds per measurement the kernel file of every component (Fortran
// unformatted: num_blk and ker0, ncoef, then ncoef pairs of 1-based block index and
// single-precision coefficient), the datum and its weight, the station and event ids
// (signed: the sign is the term's sign) and, with --loc, the (id, weight) location pairs.
// Rows of the system, in the reference's order (:101-171): one per measurement (kernel
// coefficients above the threshold, the station, event and location terms, all times the
// datum's weight; rhs = datum x weight in single precision), one damping row per unknown
// (lamb), and the smoothing operator's rows times eta for every component.  LSQR stops at
// test1 <= 1e-7, test2 <= 1e-7 or 30000 iterations (mod_LSQR.f90:153-158).  Outputs in the
// working directory as the reference names them: try.xyz and try.err (model values and
// standard errors, E12.3), try.sta and try.evt (id, term, term x weight), try.loc (--loc),
// and try.sum (fit statistics, result_evaluate :266-390).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "../../include/fwant_lsqr.h"

namespace {

[[noreturn]] void die(const std::string& msg) {
  std::fprintf(stderr, "fwant_lsqr: %s\n", msg.c_str());
  std::exit(1);
}

std::vector<std::string> words(const std::string& line) {
  std::vector<std::string> w;
  std::string t = line;
  for (char& c : t)
    if (c == ',') c = ' ';  // list-directed input separates values by blanks or commas
  std::istringstream is(t);
  for (std::string s; is >> s;) w.push_back(s);
  return w;
}

double num(const std::string& s, const char* what) {
  std::string t = s;
  for (char& c : t)
    if (c == 'd' || c == 'D') c = 'e';
  char* end = nullptr;
  const double v = std::strtod(t.c_str(), &end);
  if (end == t.c_str()) die(std::string(what) + ": not a number: " + s);
  return v;
}

// list-directed reads from standard input: values may span lines
struct Input {
  std::vector<std::string> pending;
  std::string line() {  // read(*,'(a)'): one whole record
    std::string l;
    if (!std::getline(std::cin, l)) die("standard input ended early");
    pending.clear();
    const size_t a = l.find_first_not_of(" \t\r");
    const size_t b = l.find_last_not_of(" \t\r");
    return a == std::string::npos ? "" : l.substr(a, b - a + 1);
  }
  std::vector<std::string> values(size_t n) {  // read(*,*) n values; the rest of the record is dropped
    std::vector<std::string> out;
    while (out.size() < n) {
      std::string l;
      if (!std::getline(std::cin, l)) die("standard input ended early");
      for (const std::string& w : words(l)) out.push_back(w);
    }
    out.resize(n);
    return out;
  }
};

// list-directed reads from a text file: each read starts a new record, takes values across
// records as needed and drops the rest of its last record
struct RecordReader {
  std::ifstream f;
  std::string path;
  explicit RecordReader(const std::string& p) : f(p), path(p) {}
  std::vector<std::string> values(size_t n) {
    std::vector<std::string> out;
    std::string l;
    while (out.size() < n) {
      if (!std::getline(f, l)) die(path + ": ends early");
      for (const std::string& w : words(l)) out.push_back(w);
    }
    out.resize(n);
    return out;
  }
};

// Fortran unformatted sequential records (4-byte length markers before and after, a
// negative marker continuing the record in another subrecord)
bool read_record(std::FILE* f, std::vector<unsigned char>& out) {
  out.clear();
  for (;;) {
    int32_t head = 0, tail = 0;
    if (std::fread(&head, 4, 1, f) != 1) return false;
    const bool more = head < 0;
    const uint32_t len = uint32_t(more ? -int64_t(head) : head);
    const size_t at = out.size();
    out.resize(at + len);
    if (len && std::fread(out.data() + at, 1, len, f) != len) return false;
    if (std::fread(&tail, 4, 1, f) != 1) return false;
    if (!more) return true;
  }
}

struct KernelRow {  // one kernel file
  int nblk = 0;
  std::vector<int> idx;     // 1-based block index
  std::vector<float> coef;
};

KernelRow read_kernel_file(const std::string& path) {
  std::FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) die("open kernel err: " + path);
  std::vector<unsigned char> r;
  KernelRow k;
  int32_t ncoef = 0;
  if (!read_record(f, r) || r.size() < 8) die(path + ": first record (num_blk, ker0) missing");
  std::memcpy(&k.nblk, r.data(), 4);
  if (!read_record(f, r) || r.size() < 4) die(path + ": second record (ncoef) missing");
  std::memcpy(&ncoef, r.data(), 4);
  if (ncoef < 0) die(path + ": negative ncoef");
  if (!read_record(f, r) || r.size() < size_t(ncoef) * 8) die(path + ": coefficient record short");
  std::fclose(f);
  k.idx.resize(size_t(ncoef));
  k.coef.resize(size_t(ncoef));
  for (int32_t i = 0; i < ncoef; ++i) {
    std::memcpy(&k.idx[size_t(i)], r.data() + 8 * size_t(i), 4);
    std::memcpy(&k.coef[size_t(i)], r.data() + 8 * size_t(i) + 4, 4);
  }
  return k;
}

struct Settings {
  bool loc = false;
  double lamb = 0, eta = 0, weig_sta = 0, weig_evt = 0, weig_loc = 0, ker_thres = 0, data_thres = 0;
  int num_cmp = 0, nsta = 0, nevt = 0, nloc = 0;
  std::string list, smooth;
};

// One measurement of the data list, parsed (the record's words after the kernel files)
struct Datum {
  std::vector<std::string> files;
  float rhs = 0, weig = 0;
  std::vector<int> sta, evt, loc_id;
  std::vector<double> loc_w;
};

bool parse_datum(const std::string& raw, const Settings& s, Datum* d) {
  std::string t = raw.substr(0, std::min<size_t>(raw.size(), 300));
  const size_t a = t.find_first_not_of(" \t\r");
  if (a == std::string::npos) return false;  // blank record
  t = t.substr(a);
  if (t[0] == '#') return false;
  const auto w = words(t);
  size_t need = size_t(s.num_cmp) + 2 + size_t(s.nsta) + size_t(s.nevt) + 2 * size_t(s.nloc);
  if (w.size() < need) die(s.list + ": a measurement needs " + std::to_string(need) + " words: " + t);
  size_t p = 0;
  d->files.assign(w.begin(), w.begin() + s.num_cmp);
  p = size_t(s.num_cmp);
  d->rhs = float(num(w[p++], "datum"));
  d->weig = float(num(w[p++], "weight"));
  d->sta.clear();
  d->evt.clear();
  d->loc_id.clear();
  d->loc_w.clear();
  for (int k = 0; k < s.nsta; ++k) d->sta.push_back(int(num(w[p++], "station id")));
  for (int k = 0; k < s.nevt; ++k) d->evt.push_back(int(num(w[p++], "event id")));
  for (int k = 0; k < s.nloc; ++k) {
    d->loc_id.push_back(int(num(w[p++], "location id")));
    d->loc_w.push_back(num(w[p++], "location weight"));
  }
  return true;
}

double fsign(double a, double b) { return b >= 0.0 ? std::fabs(a) : -std::fabs(a); }

// A measurement's row without the datum weight (coefficients above ker_thres with their
// component offsets, then the station, event and location terms), 0-based columns.
void datum_row(const Datum& d, const std::vector<KernelRow>& ks, const Settings& s, long long num_mval,
               long long num_sta, long long num_evt, std::vector<int>* cols, std::vector<double>* coefs) {
  cols->clear();
  coefs->clear();
  for (size_t k = 0; k < ks.size(); ++k)
    for (size_t i = 0; i < ks[k].idx.size(); ++i) {
      const double tmp = double(ks[k].coef[i]);
      if (std::fabs(tmp) > s.ker_thres) {
        cols->push_back(int(ks[k].idx[i] + (long long)ks[k].nblk * (long long)k - 1));
        coefs->push_back(tmp);
      }
    }
  for (int id : d.sta) {
    cols->push_back(int(num_mval + std::abs(id) - 1));
    coefs->push_back(fsign(s.weig_sta, double(id)));
  }
  for (int id : d.evt) {
    cols->push_back(int(num_mval + num_sta + std::abs(id) - 1));
    coefs->push_back(fsign(s.weig_evt, double(id)));
  }
  for (size_t k = 0; k < d.loc_id.size(); ++k) {
    cols->push_back(int(num_mval + num_sta + num_evt + d.loc_id[k] - 1));
    coefs->push_back(d.loc_w[k] * s.weig_loc);
  }
}

// Fortran E12.3 (0.ddd E+xx) and F10.5 / I5 fields
std::string fmt_e12_3(double v) {
  char b[64];
  if (v == 0.0 || !std::isfinite(v)) {
    if (!std::isfinite(v)) return std::string(12, '*');
    std::snprintf(b, sizeof(b), "%12s", std::signbit(v) ? "-0.000E+00" : "0.000E+00");
    return b;
  }
  std::snprintf(b, sizeof(b), "%.2e", v);  // d.dde+xx: the same three significant digits
  const std::string m = b;
  const size_t e = m.find('e');
  const int ex = std::atoi(m.c_str() + e + 1) + 1;
  std::string digits;
  for (size_t i = 0; i < e; ++i)
    if (m[i] >= '0' && m[i] <= '9') digits.push_back(m[i]);
  char out[64];
  if (std::abs(ex) <= 99)
    std::snprintf(out, sizeof(out), "%s0.%sE%c%02d", v < 0 ? "-" : "", digits.c_str(), ex < 0 ? '-' : '+', std::abs(ex));
  else
    std::snprintf(out, sizeof(out), "%s0.%s%c%03d", v < 0 ? "-" : "", digits.c_str(), ex < 0 ? '-' : '+', std::abs(ex));
  std::snprintf(b, sizeof(b), "%12s", out);
  return std::strlen(b) > 12 ? std::string(12, '*') : std::string(b);
}
std::string fmt_f(double v, int w, int d) {
  char b[128];
  std::snprintf(b, sizeof(b), "%*.*f", w, d, v);
  return int(std::strlen(b)) > w ? std::string(size_t(w), '*') : std::string(b);
}
std::string fmt_i5(long long v) {
  char b[64];
  std::snprintf(b, sizeof(b), "%5lld", v);
  return std::strlen(b) > 5 ? std::string(5, '*') : std::string(b);
}

}  // namespace

int main(int argc, char** argv) {
  Settings s;
  int device = 0;
  std::string dump;  // write the assembled system (PREFIX.rp .col .val .rhs) and stop
  for (int a = 1; a < argc; ++a) {
    const std::string t = argv[a];
    if (t == "--loc") s.loc = true;
    else if (t == "--device" && a + 1 < argc) device = std::atoi(argv[++a]);
    else if (t == "--dump-system" && a + 1 < argc) dump = argv[++a];
    else die("usage: fwant_lsqr [--loc] [--device N] [--dump-system PREFIX] < answers");
  }
  Input in;
  const int imultis = int(num(in.values(1)[0], "mode"));
  if (imultis != 1) die("only Simple damping valid");
  auto two = [&](const char* what) {
    const auto v = in.values(2);
    return std::make_pair(num(v[0], what), num(v[1], what));
  };
  if (!s.loc) {
    std::tie(s.lamb, s.eta) = two("damping and smoothing");
    s.num_cmp = int(num(in.values(1)[0], "components"));
    auto p = two("station terms");
    s.nsta = int(p.first), s.weig_sta = p.second;
    p = two("event terms");
    s.nevt = int(p.first), s.weig_evt = p.second;
    s.list = in.line();
    s.smooth = in.line();
  } else {
    s.list = in.line();
    s.smooth = in.line();
    s.num_cmp = int(num(in.values(1)[0], "components"));
    auto p = two("station terms");
    s.nsta = int(p.first), s.weig_sta = p.second;
    p = two("event terms");
    s.nevt = int(p.first), s.weig_evt = p.second;
    p = two("location terms");
    s.nloc = int(p.first), s.weig_loc = p.second;
    std::tie(s.lamb, s.eta) = two("damping and smoothing");
  }
  std::tie(s.ker_thres, s.data_thres) = two("kernel and measurement thresholds");
  if (s.num_cmp < 1 || s.nsta < 0 || s.nevt < 0 || s.nloc < 0) die("component and term counts must be >= 0");

  // pass 1 (init_data_damp, :191-265): sizes; nblk is the last kernel file's
  std::vector<std::string> records;
  {
    std::ifstream f(s.list);
    if (!f) die("fnm_list open err: " + s.list);
    for (std::string l; std::getline(f, l);) records.push_back(l);
  }
  int nblk = 0;
  long long max_st = 0, max_ev = 0, max_lo = 0, ndat = 0;
  Datum d;
  for (const std::string& r : records) {
    if (!parse_datum(r, s, &d)) continue;
    ++ndat;
    for (const std::string& fn : d.files) nblk = read_kernel_file(fn).nblk;
    for (int id : d.sta) max_st = std::max<long long>(max_st, std::abs(id));
    for (int id : d.evt) max_ev = std::max<long long>(max_ev, std::abs(id));
    for (int id : d.loc_id) max_lo = std::max<long long>(max_lo, std::abs(id));
  }
  if (ndat == 0) die(s.list + ": no measurements");
  const long long num_mval = (long long)nblk * s.num_cmp;
  const long long num_xval = num_mval + max_st + max_ev + max_lo;
  if (num_xval > 0x7fffffffLL) die("more than 2^31 unknowns");

  // the system's rows
  std::vector<long long> rp(1, 0);
  std::vector<int> col;
  std::vector<double> val, rhs;
  float rmin = 1.e7f, rmax = -1.e7f, rwmin = 1.e7f, rwmax = -1.e7f;
  std::vector<int> cols;
  std::vector<double> coefs;
  auto add_row = [&](const std::vector<int>& c, const std::vector<double>& v, double b) {  // lldrow
    if (c.empty()) return;
    for (int j : c)
      if (j < 0 || j >= num_xval) die("column index outside the unknowns (a block or term id out of range)");
    col.insert(col.end(), c.begin(), c.end());
    val.insert(val.end(), v.begin(), v.end());
    rp.push_back((long long)col.size());
    rhs.push_back(b);
  };
  for (const std::string& r : records) {
    if (!parse_datum(r, s, &d)) continue;
    std::vector<KernelRow> ks;
    for (const std::string& fn : d.files) ks.push_back(read_kernel_file(fn));
    if (std::fabs(d.rhs) > s.data_thres) {
      std::printf(" omit large rhs= %g\n", double(d.rhs));
      continue;
    }
    datum_row(d, ks, s, num_mval, max_st, max_ev, &cols, &coefs);
    rmin = std::min(rmin, d.rhs);
    rmax = std::max(rmax, d.rhs);
    for (double& c : coefs) c = c * double(d.weig);
    const float rw = d.rhs * d.weig;  // single precision, as the reference
    rwmin = std::min(rwmin, rw);
    rwmax = std::max(rwmax, rw);
    add_row(cols, coefs, double(rw));
  }
  const long long ndata_rows = (long long)rhs.size();
  for (long long i = 0; i < num_xval; ++i) add_row({int(i)}, {s.lamb}, 0.0);  // damping
  // smoothing operator (:155-169): num_blk nrow nbd nel, then per row ncoef, its indices,
  // its values; the component offset is this file's num_blk
  std::vector<std::vector<int>> sm_idx;
  std::vector<std::vector<float>> sm_coef;
  long long sm_nblk = 0;
  {
    RecordReader f(s.smooth);
    if (!f.f) die("open smoothing file err: " + s.smooth);
    const auto head = f.values(4);
    sm_nblk = (long long)num(head[0], "smoothing num_blk");
    const long long nrow_sm = (long long)num(head[1], "smoothing rows");
    for (long long n = 0; n < nrow_sm; ++n) {
      std::string l;
      // ncoef first, then the rest of the same read
      std::vector<std::string> v;
      while (v.empty()) {
        if (!std::getline(f.f, l)) die(s.smooth + ": ends early");
        v = words(l);
      }
      const int nc = int(num(v[0], "smoothing ncoef"));
      if (nc < 0) die(s.smooth + ": negative ncoef");
      while (v.size() < size_t(1 + 2 * nc)) {
        if (!std::getline(f.f, l)) die(s.smooth + ": ends early");
        for (const std::string& w : words(l)) v.push_back(w);
      }
      std::vector<int> ix(static_cast<size_t>(nc));
      std::vector<float> cf(static_cast<size_t>(nc));
      for (int i = 0; i < nc; ++i) ix[size_t(i)] = int(num(v[size_t(1 + i)], "smoothing index"));
      for (int i = 0; i < nc; ++i) cf[size_t(i)] = float(num(v[size_t(1 + nc + i)], "smoothing coefficient"));
      for (int k = 0; k < s.num_cmp; ++k) {
        cols.clear();
        coefs.clear();
        for (int i = 0; i < nc; ++i) {
          cols.push_back(int(ix[size_t(i)] + (long long)k * sm_nblk - 1));
          coefs.push_back(double(cf[size_t(i)]) * s.eta);
        }
        add_row(cols, coefs, 0.0);
      }
      sm_idx.push_back(std::move(ix));
      sm_coef.push_back(std::move(cf));
    }
  }
  const long long nrow = (long long)rhs.size();
  std::printf(" # of dat, mval, xval: %lld %lld %lld\n # of row, nel: %lld %lld\n", ndata_rows, num_mval, num_xval,
              nrow, (long long)col.size());
  std::printf(" rhs_min,rhs_max\n %g %g\n rhs_min_weig,rhs_max_weig\n %g %g\n", double(rmin), double(rmax),
              double(rwmin), double(rwmax));
  if (!dump.empty()) {
    auto put = [&](const std::string& ext, const void* p, size_t bytes) {
      std::FILE* f = std::fopen((dump + ext).c_str(), "wb");
      if (!f || std::fwrite(p, 1, bytes, f) != bytes) die("cannot write " + dump + ext);
      std::fclose(f);
    };
    put(".rp", rp.data(), rp.size() * sizeof(long long));
    put(".col", col.data(), col.size() * sizeof(int));
    put(".val", val.data(), val.size() * sizeof(double));
    put(".rhs", rhs.data(), rhs.size() * sizeof(double));
    std::printf(" system written to %s.{rp,col,val,rhs}: %lld rows, %lld columns\n", dump.c_str(), nrow, num_xval);
    return 0;
  }

  // slsqr + lgtsol on the device
  fwant_lsqr* L = nullptr;
  fwant_status rc = fwant_lsqr_create(nrow, num_xval, rp.data(), col.data(), val.data(), rhs.data(), device, &L);
  if (rc != FWANT_OK) die("lsqr_create failed (status " + std::to_string(int(rc)) + ")");
  long long itct = 0;
  if (fwant_lsqr_solve(L, 1.0e-7, 1.0e-7, 30000, &itct) != FWANT_OK) die(fwant_lsqr_last_error(L));
  std::vector<double> mval(static_cast<size_t>(num_xval)), errx(static_cast<size_t>(num_xval));
  if (fwant_lsqr_solution(L, num_xval, mval.data(), errx.data()) != FWANT_OK) die(fwant_lsqr_last_error(L));
  double info[6];
  fwant_lsqr_info(L, info);
  double ms = 0.0;
  fwant_lsqr_last_solve_ms(L, &ms);
  fwant_lsqr_destroy(L);
  std::printf(" iter., test1, test2: %lld %lld %lld %lld %.4e %.4e %.4e\n", itct, nrow, num_xval, (long long)col.size(),
              info[2], info[3], info[4]);
  std::printf(" solve: %.3f ms on the device\n", ms);

  // export_result (:392-420)
  {
    std::FILE* f = std::fopen("try.xyz", "w");
    std::FILE* g = std::fopen("try.err", "w");
    if (!f || !g) die("cannot write try.xyz / try.err");
    for (long long i = 0; i < num_mval; ++i) {
      std::fprintf(f, "%s\n", fmt_e12_3(mval[size_t(i)]).c_str());
      std::fprintf(g, "%s\n", fmt_e12_3(errx[size_t(i)]).c_str());
    }
    std::fclose(f);
    std::fclose(g);
    f = std::fopen("try.sta", "w");
    g = std::fopen("try.evt", "w");
    if (!f || !g) die("cannot write try.sta / try.evt");
    for (long long i = 1; i <= max_st; ++i) {
      const double m = mval[size_t(num_mval + i - 1)];
      std::fprintf(f, "%s%s%s\n", fmt_i5(i).c_str(), fmt_f(m, 10, 5).c_str(), fmt_f(m * s.weig_sta, 10, 5).c_str());
    }
    for (long long i = 1; i <= max_ev; ++i) {
      const double m = mval[size_t(num_mval + max_st + i - 1)];
      std::fprintf(g, "%s%s%s\n", fmt_i5(i).c_str(), fmt_f(m, 10, 5).c_str(), fmt_f(m * s.weig_evt, 10, 5).c_str());
    }
    std::fclose(f);
    std::fclose(g);
    if (s.loc) {
      f = std::fopen("try.loc", "w");
      if (!f) die("cannot write try.loc");
      for (long long i = 1; i <= max_lo; ++i)
        std::fprintf(f, "%s%s\n", fmt_i5(i).c_str(), fmt_f(mval[size_t(num_mval + max_st + max_ev + i - 1)], 10, 5).c_str());
      std::fclose(f);
    }
  }
  // result_evaluate (:266-390): fits without and with the data weights, smoothness, model
  // statistics
  double fit = 0, dvar = 0, fit_w = 0, dvar_w = 0, vmin_loc = 1.e7, vmax_loc = -1.e7;
  long long nd = 0;
  for (const std::string& r : records) {
    if (!parse_datum(r, s, &d)) continue;
    std::vector<KernelRow> ks;
    for (const std::string& fn : d.files) ks.push_back(read_kernel_file(fn));
    if (std::fabs(d.rhs) > s.data_thres) continue;
    ++nd;
    const float rw = d.rhs * d.weig;
    dvar = dvar + double(d.rhs) * double(d.rhs);
    dvar_w = dvar_w + double(rw) * double(rw);
    datum_row(d, ks, s, num_mval, max_st, max_ev, &cols, &coefs);
    double tmp = 0.0;
    for (size_t i = 0; i < cols.size(); ++i) tmp = tmp + coefs[i] * mval[size_t(cols[i])];
    for (size_t k = 0; k < d.loc_id.size(); ++k) {
      const double t = mval[size_t(num_mval + max_st + max_ev + d.loc_id[k] - 1)] * d.loc_w[k] * s.weig_loc;
      vmin_loc = std::min(t, vmin_loc);
      vmax_loc = std::max(t, vmax_loc);
    }
    const double tmp_w = tmp * double(d.weig);
    fit = fit + (tmp - double(d.rhs)) * (tmp - double(d.rhs));
    fit_w = fit_w + (tmp_w - double(rw)) * (tmp_w - double(rw));
  }
  const double kai2 = fit_w / double(nd);
  fit = (1.0 - fit / dvar) * 100.0;
  fit_w = (1.0 - fit_w / dvar_w) * 100.0;
  double smocov = 0.0;
  for (size_t n = 0; n < sm_idx.size(); ++n)
    for (int k = 0; k < s.num_cmp; ++k) {
      double t = 0.0;
      for (size_t i = 0; i < sm_idx[n].size(); ++i)
        t = t + double(sm_coef[n][i]) * mval[size_t(sm_idx[n][i] + (long long)k * sm_nblk - 1)];
      smocov = smocov + t * t;
    }
  smocov = std::sqrt(smocov / double(num_mval));
  double mean = 0, cov = 0, norm = 0, vmin = 1.e7, vmax = -1.e7;
  double vmin_sta = 1.e7, vmax_sta = -1.e7, vmin_evt = 1.e7, vmax_evt = -1.e7;
  for (long long j = 0; j < num_mval; ++j) {
    cov = cov + errx[size_t(j)] * errx[size_t(j)];
    norm = norm + mval[size_t(j)] * mval[size_t(j)];
    mean = mean + mval[size_t(j)];
    vmin = std::min(mval[size_t(j)], vmin);
    vmax = std::max(mval[size_t(j)], vmax);
  }
  for (long long j = num_mval; j < num_mval + max_st; ++j) {
    vmin_sta = std::min(mval[size_t(j)] * s.weig_sta, vmin_sta);
    vmax_sta = std::max(mval[size_t(j)] * s.weig_sta, vmax_sta);
  }
  for (long long j = num_mval + max_st; j < num_mval + max_st + max_ev; ++j) {
    vmin_evt = std::min(mval[size_t(j)] * s.weig_evt, vmin_evt);
    vmax_evt = std::max(mval[size_t(j)] * s.weig_evt, vmax_evt);
  }
  norm = std::sqrt(norm / double(num_mval));
  cov = std::sqrt(cov / double(num_mval));
  mean = mean / double(num_mval);
  std::FILE* f = std::fopen("try.sum", "w");
  if (!f) die("cannot write try.sum");
  auto kv = [&](const char* k, double v) { std::fprintf(f, " %s = %24.15E\n", k, v); };
  std::fprintf(f, " mode = Simple\n");
  kv("damping", s.lamb);
  kv("smoothing", s.eta);
  kv("percent of data_var reduction", fit);
  kv("percent of data_var reduction w weight", fit_w);
  kv("kai^2", kai2 * double(nd));
  std::fprintf(f, " number of data = %lld\n", nd);
  kv("kai^2/N", kai2);
  kv("error_variance (model_var?)", cov);
  kv("smooth_norm", smocov);
  kv("model_norm (model_var?)", norm);
  kv("model_mean", mean);
  kv("model_min", vmin);
  kv("model_max", vmax);
  kv("station_term_min", vmin_sta);
  kv("station_term_max", vmax_sta);
  kv("event_term_min", vmin_evt);
  kv("event_term_max", vmax_evt);
  if (s.loc) {
    kv("location_term_min", vmin_loc);
    kv("location_term_max", vmax_loc);
  }
  std::fclose(f);
  std::printf(" damping, smoothing, data_var_reduc, model_norm\n %g %g %g %g\n", s.lamb, s.eta, fit, norm);
  return 0;
}
