// NetCDF classic-format reader and writer (see netcdf3.h).
#include "netcdf3.h"

#include <cstring>

namespace nc3 {

namespace {
constexpr uint32_t TAG_DIMENSION = 0x0A, TAG_VARIABLE = 0x0B, TAG_ATTRIBUTE = 0x0C;

uint64_t pad4(uint64_t n) { return (n + 3) & ~uint64_t(3); }

// big-endian scalar encode / decode
void put_be(std::vector<unsigned char>& b, uint64_t v, int bytes) {
  for (int i = bytes - 1; i >= 0; --i) b.push_back(static_cast<unsigned char>(v >> (8 * i)));
}
uint64_t get_be(const unsigned char* p, int bytes) {
  uint64_t v = 0;
  for (int i = 0; i < bytes; ++i) v = (v << 8) | p[i];
  return v;
}
double decode(const unsigned char* p, int type) {
  switch (type) {
    case NC_BYTE: return double(int8_t(p[0]));
    case NC_CHAR: return double(p[0]);
    case NC_SHORT: return double(int16_t(uint16_t(get_be(p, 2))));
    case NC_INT: return double(int32_t(uint32_t(get_be(p, 4))));
    case NC_FLOAT: {
      const uint32_t u = uint32_t(get_be(p, 4));
      float f;
      std::memcpy(&f, &u, 4);
      return double(f);
    }
    default: {
      const uint64_t u = get_be(p, 8);
      double d;
      std::memcpy(&d, &u, 8);
      return d;
    }
  }
}
void encode(std::vector<unsigned char>& b, double v, int type) {
  switch (type) {
    case NC_BYTE: b.push_back(static_cast<unsigned char>(int8_t(v))); break;
    case NC_CHAR: b.push_back(static_cast<unsigned char>(v)); break;
    case NC_SHORT: put_be(b, uint16_t(int16_t(v)), 2); break;
    case NC_INT: put_be(b, uint32_t(int32_t(v)), 4); break;
    case NC_FLOAT: {
      const float f = float(v);
      uint32_t u;
      std::memcpy(&u, &f, 4);
      put_be(b, u, 4);
      break;
    }
    default: {
      uint64_t u;
      std::memcpy(&u, &v, 8);
      put_be(b, u, 8);
    }
  }
}

// sequential header parser over a byte buffer
struct Cursor {
  const std::vector<unsigned char>& b;
  size_t o = 0;
  bool ok = true;
  explicit Cursor(const std::vector<unsigned char>& buf) : b(buf) {}
  uint64_t u(int bytes) {
    if (o + bytes > b.size()) { ok = false; return 0; }
    const uint64_t v = get_be(&b[o], bytes);
    o += bytes;
    return v;
  }
  std::string name() {
    const uint64_t n = u(4);
    if (!ok || o + n > b.size() || n > (1u << 20)) { ok = false; return ""; }
    std::string s(reinterpret_cast<const char*>(&b[o]), size_t(n));
    o += pad4(n);
    return s;
  }
  bool att_list(std::vector<Att>& out) {
    const uint64_t tag = u(4), n = u(4);
    if (!ok) return false;
    if (tag == 0 && n == 0) return true;
    if (tag != TAG_ATTRIBUTE || n > (1u << 20)) return ok = false;
    for (uint64_t i = 0; i < n && ok; ++i) {
      Att a;
      a.name = name();
      a.type = int(u(4));
      const uint64_t cnt = u(4);
      const int sz = type_size(a.type);
      if (!ok || sz == 0 || o + cnt * sz > b.size()) return ok = false;
      if (a.type == NC_CHAR) a.text.assign(reinterpret_cast<const char*>(&b[o]), size_t(cnt));
      else
        for (uint64_t e = 0; e < cnt; ++e) a.num.push_back(decode(&b[o + e * sz], a.type));
      o += pad4(cnt * sz);
      out.push_back(a);
    }
    return ok;
  }
};
}  // namespace

int type_size(int type) {
  switch (type) {
    case NC_BYTE: case NC_CHAR: return 1;
    case NC_SHORT: return 2;
    case NC_INT: case NC_FLOAT: return 4;
    case NC_DOUBLE: return 8;
    default: return 0;
  }
}

Reader::~Reader() {
  if (fp_) std::fclose(fp_);
}

bool Reader::open(const std::string& path, std::string* err) {
  fp_ = std::fopen(path.c_str(), "rb");
  if (!fp_) { *err = "cannot open " + path; return false; }
  // the header is at most a few MB for any file of the solver: read a generous prefix
  std::vector<unsigned char> b(1 << 22);
  b.resize(std::fread(b.data(), 1, b.size(), fp_));
  Cursor c(b);
  const uint64_t magic = c.u(4);
  int version = 0;
  if (magic == 0x43444601ULL) version = 1;
  else if (magic == 0x43444602ULL) version = 2;
  else { *err = path + ": not a NetCDF classic file"; return false; }
  numrecs_ = c.u(4);
  // dimensions
  uint64_t tag = c.u(4), n = c.u(4);
  if (!(tag == 0 && n == 0)) {
    if (tag != TAG_DIMENSION || n > (1u << 20)) c.ok = false;
    for (uint64_t i = 0; i < n && c.ok; ++i) {
      Dim d;
      d.name = c.name();
      d.len = c.u(4);
      dims.push_back(d);
    }
  }
  c.att_list(gatts);
  // variables
  tag = c.u(4);
  n = c.u(4);
  if (c.ok && !(tag == 0 && n == 0)) {
    if (tag != TAG_VARIABLE || n > (1u << 20)) c.ok = false;
    for (uint64_t i = 0; i < n && c.ok; ++i) {
      Var v;
      v.name = c.name();
      const uint64_t nd = c.u(4);
      if (nd > 64) { c.ok = false; break; }
      for (uint64_t e = 0; e < nd; ++e) {
        const uint64_t id = c.u(4);
        if (id >= dims.size()) c.ok = false;
        v.dims.push_back(int(id));
      }
      c.att_list(v.atts);
      v.type = int(c.u(4));
      v.vsize = c.u(4);
      v.begin = c.u(version == 2 ? 8 : 4);
      v.record = !v.dims.empty() && c.ok && dims[v.dims[0]].len == 0;
      if (type_size(v.type) == 0) c.ok = false;
      vars.push_back(v);
    }
  }
  if (!c.ok) { *err = path + ": damaged NetCDF header"; return false; }
  // record size: the record slices of all record variables; with a single record
  // variable the slices follow each other unpadded
  int nrec = 0;
  uint64_t slice = 0;
  recsize_ = 0;
  for (const Var& v : vars)
    if (v.record) {
      ++nrec;
      recsize_ += v.vsize;
      slice = count(v) / (numrecs_ ? numrecs_ : 1) * type_size(v.type);
    }
  if (nrec == 1) recsize_ = slice;
  return true;
}

const Dim* Reader::dim(const std::string& name) const {
  for (const Dim& d : dims)
    if (d.name == name) return &d;
  return nullptr;
}
const Var* Reader::var(const std::string& name) const {
  for (const Var& v : vars)
    if (v.name == name) return &v;
  return nullptr;
}
const Att* Reader::gatt(const std::string& name) const {
  for (const Att& a : gatts)
    if (a.name == name) return &a;
  return nullptr;
}

uint64_t Reader::count(const Var& v) const {
  uint64_t n = 1;
  for (int id : v.dims) n *= dims[id].len == 0 ? numrecs_ : dims[id].len;
  return n;
}

bool Reader::read_raw(const Var& v, std::vector<double>* out, std::string* err) const {
  const int sz = type_size(v.type);
  const uint64_t n = count(v);
  out->resize(size_t(n));
  const uint64_t per = v.record ? (numrecs_ ? n / numrecs_ : 0) : n;  // elements per record
  const uint64_t nr = v.record ? numrecs_ : 1;
  std::vector<unsigned char> buf(size_t(per * sz));
  for (uint64_t r = 0; r < nr; ++r) {
    const uint64_t off = v.begin + r * recsize_;
    if (std::fseek(fp_, long(off), SEEK_SET) != 0 || std::fread(buf.data(), 1, buf.size(), fp_) != buf.size()) {
      *err = "truncated data of variable " + v.name;
      return false;
    }
    for (uint64_t e = 0; e < per; ++e) (*out)[size_t(r * per + e)] = decode(&buf[size_t(e * sz)], v.type);
  }
  return true;
}

bool Reader::read(const std::string& name, std::vector<double>* out, std::string* err) const {
  const Var* v = var(name);
  if (!v) { *err = "no variable " + name; return false; }
  return read_raw(*v, out, err);
}
bool Reader::read(const std::string& name, std::vector<float>* out, std::string* err) const {
  std::vector<double> d;
  if (!read(name, &d, err)) return false;
  out->assign(d.begin(), d.end());
  return true;
}
bool Reader::read(const std::string& name, std::vector<int>* out, std::string* err) const {
  std::vector<double> d;
  if (!read(name, &d, err)) return false;
  out->resize(d.size());
  for (size_t i = 0; i < d.size(); ++i) (*out)[i] = int(d[i]);
  return true;
}

namespace {
// Element offsets of a hyperslab: calls row(file_offset_of_first, slab_index_of_first) for
// every run along the last dimension (count elements stride apart).
template <typename F>
bool for_rows(const Reader& r, const Var& v, uint64_t numrecs, uint64_t recsize, const std::vector<uint64_t>& start,
              const std::vector<uint64_t>& cnt, const std::vector<uint64_t>& stride, std::string* err, F row) {
  const size_t nd = v.dims.size();
  if (nd == 0 || start.size() != nd || cnt.size() != nd || stride.size() != nd) {
    *err = "variable " + v.name + ": slab rank differs from the variable's";
    return false;
  }
  const int sz = type_size(v.type);
  std::vector<uint64_t> len(nd), pitch(nd);
  for (size_t d = 0; d < nd; ++d) {
    len[d] = r.dims[v.dims[d]].len == 0 ? numrecs : r.dims[v.dims[d]].len;
    if (cnt[d] == 0) return true;
    if (stride[d] == 0 || start[d] + (cnt[d] - 1) * stride[d] >= len[d]) {
      *err = "variable " + v.name + ": slab outside dimension " + r.dims[v.dims[d]].name;
      return false;
    }
  }
  // byte pitch of each dimension
  uint64_t p = uint64_t(sz);
  for (size_t d = nd; d-- > 0;) {
    pitch[d] = p;
    if (!(d == 0 && v.record)) p *= len[d];
  }
  if (v.record) pitch[0] = recsize;
  std::vector<uint64_t> idx(nd - 1, 0);
  uint64_t slab = 0;
  for (;;) {
    uint64_t off = v.begin + start[nd - 1] * pitch[nd - 1];
    for (size_t d = 0; d + 1 < nd; ++d) off += (start[d] + idx[d] * stride[d]) * pitch[d];
    if (!row(off, slab)) return false;
    slab += cnt[nd - 1];
    size_t d = nd - 1;
    while (d > 0) {
      --d;
      if (++idx[d] < cnt[d]) break;
      idx[d] = 0;
      if (d == 0) return true;
    }
    if (nd == 1) return true;
  }
}
}  // namespace

bool Reader::read_slab(const std::string& name, const std::vector<uint64_t>& start, const std::vector<uint64_t>& cnt,
                       const std::vector<uint64_t>& stride, std::vector<float>* out, std::string* err) const {
  const Var* v = var(name);
  if (!v) { *err = "no variable " + name; return false; }
  uint64_t total = 1;
  for (uint64_t c : cnt) total *= c;
  out->assign(size_t(total), 0.0f);
  if (total == 0) return true;
  const int sz = type_size(v->type);
  const uint64_t n = cnt.back(), st = stride.back(), span = (n - 1) * st + 1;
  std::vector<unsigned char> buf(size_t(span * sz));
  return for_rows(*this, *v, numrecs_, recsize_, start, cnt, stride, err, [&](uint64_t off, uint64_t slab) {
    if (std::fseek(fp_, long(off), SEEK_SET) != 0 || std::fread(buf.data(), 1, buf.size(), fp_) != buf.size()) {
      *err = "truncated data of variable " + v->name;
      return false;
    }
    for (uint64_t e = 0; e < n; ++e) (*out)[size_t(slab + e)] = float(decode(&buf[size_t(e * st * sz)], v->type));
    return true;
  });
}

bool update_slab(const std::string& path, const std::string& name, const std::vector<uint64_t>& start,
                 const std::vector<uint64_t>& cnt, const std::vector<uint64_t>& stride, const float* data,
                 std::string* err) {
  Reader r;
  if (!r.open(path, err)) return false;
  const Var* v = r.var(name);
  if (!v) { *err = path + ": no variable " + name; return false; }
  if (v->type != NC_FLOAT || v->record) { *err = path + ": " + name + " is not a fixed-size float variable"; return false; }
  FILE* f = std::fopen(path.c_str(), "r+b");
  if (!f) { *err = "cannot open " + path + " for writing"; return false; }
  const uint64_t n = cnt.empty() ? 0 : cnt.back(), st = stride.empty() ? 1 : stride.back(), span = n ? (n - 1) * st + 1 : 0;
  std::vector<unsigned char> buf(size_t(span * 4)), one;
  const bool ok = for_rows(r, *v, r.numrecs_, r.recsize_, start, cnt, stride, err, [&](uint64_t off, uint64_t slab) {
    if (std::fseek(f, long(off), SEEK_SET) != 0 || std::fread(buf.data(), 1, buf.size(), f) != buf.size()) {
      *err = path + ": truncated data of variable " + name;
      return false;
    }
    for (uint64_t e = 0; e < n; ++e) {
      one.clear();
      encode(one, double(data[slab + e]), NC_FLOAT);
      std::memcpy(&buf[size_t(e * st * 4)], one.data(), 4);
    }
    if (std::fseek(f, long(off), SEEK_SET) != 0 || std::fwrite(buf.data(), 1, buf.size(), f) != buf.size()) {
      *err = path + ": write failed";
      return false;
    }
    return true;
  });
  if (std::fclose(f) != 0 && ok) { *err = path + ": write failed"; return false; }
  return ok;
}

// ---- writer ------------------------------------------------------------------------------
int Writer::add_dim(const std::string& name, uint64_t len) {
  dims_.push_back(Dim{name, len});
  return int(dims_.size()) - 1;
}
void Writer::add_gatt_text(const std::string& name, const std::string& text) {
  Att a;
  a.name = name;
  a.type = NC_CHAR;
  a.text = text;
  gatts_.push_back(a);
}
void Writer::add_gatt(const std::string& name, int type, const std::vector<double>& values) {
  Att a;
  a.name = name;
  a.type = type;
  a.num = values;
  gatts_.push_back(a);
}
int Writer::add_var(const std::string& name, int type, const std::vector<int>& dims,
                    const std::vector<double>& data) {
  Var v;
  v.name = name;
  v.type = type;
  v.dims = dims;
  v.record = !dims.empty() && dims_[dims[0]].len == 0;
  vars_.push_back(v);
  std::vector<unsigned char> b;
  b.reserve(data.size() * type_size(type));
  for (double x : data) encode(b, x, type);
  data_.push_back(std::move(b));
  return int(vars_.size()) - 1;
}
int Writer::add_var_f(const std::string& name, const std::vector<int>& dims, const float* data, size_t n) {
  Var v;
  v.name = name;
  v.type = NC_FLOAT;
  v.dims = dims;
  v.record = !dims.empty() && dims_[dims[0]].len == 0;
  vars_.push_back(v);
  std::vector<unsigned char> b;
  b.reserve(n * 4);
  for (size_t i = 0; i < n; ++i) {
    uint32_t u;
    std::memcpy(&u, &data[i], 4);
    put_be(b, u, 4);
  }
  data_.push_back(std::move(b));
  return int(vars_.size()) - 1;
}

int Writer::add_var_i(const std::string& name, const std::vector<int>& dims, const int* data, size_t n) {
  Var v;
  v.name = name;
  v.type = NC_INT;
  v.dims = dims;
  v.record = !dims.empty() && dims_[dims[0]].len == 0;
  vars_.push_back(v);
  std::vector<unsigned char> b;
  b.reserve(n * 4);
  for (size_t i = 0; i < n; ++i) put_be(b, uint32_t(data[i]), 4);
  data_.push_back(std::move(b));
  return int(vars_.size()) - 1;
}
int Writer::add_var_c(const std::string& name, const std::vector<int>& dims, const char* data, size_t n) {
  Var v;
  v.name = name;
  v.type = NC_CHAR;
  v.dims = dims;
  v.record = !dims.empty() && dims_[dims[0]].len == 0;
  vars_.push_back(v);
  data_.emplace_back(reinterpret_cast<const unsigned char*>(data), reinterpret_cast<const unsigned char*>(data) + n);
  return int(vars_.size()) - 1;
}

bool Writer::write(const std::string& path, std::string* err) const {
  // sizes: fixed variables whole, record variables one record slice
  std::vector<Var> vars = vars_;
  uint64_t fixed_total = 0, rec_total = 0;
  int nrec = 0;
  for (size_t i = 0; i < vars.size(); ++i) {
    Var& v = vars[i];
    uint64_t elems = 1;
    for (size_t d = v.record ? 1 : 0; d < v.dims.size(); ++d) elems *= dims_[v.dims[d]].len;
    const uint64_t bytes = elems * type_size(v.type);
    v.vsize = pad4(bytes);
    const uint64_t have = data_[i].size(), want = v.record ? bytes * numrecs_ : bytes;
    if (have != want) {
      *err = "variable " + v.name + ": data size does not match its dimensions";
      return false;
    }
    if (v.record) { rec_total += v.vsize; ++nrec; }
    else fixed_total += v.vsize;
  }
  uint64_t recsize = rec_total;
  if (nrec == 1)
    for (const Var& v : vars)
      if (v.record) recsize = data_[&v - &vars[0]].size() / (numrecs_ ? numrecs_ : 1);
  // header (written twice: first to learn its size, then with the offsets)
  auto header = [&](int version, std::vector<Var>& vs) {
    std::vector<unsigned char> h;
    put_be(h, version == 2 ? 0x43444602ULL : 0x43444601ULL, 4);
    put_be(h, numrecs_, 4);
    auto name = [&](const std::string& s) {
      put_be(h, s.size(), 4);
      h.insert(h.end(), s.begin(), s.end());
      while (h.size() % 4) h.push_back(0);
    };
    auto atts = [&](const std::vector<Att>& as) {
      if (as.empty()) { put_be(h, 0, 4); put_be(h, 0, 4); return; }
      put_be(h, TAG_ATTRIBUTE, 4);
      put_be(h, as.size(), 4);
      for (const Att& a : as) {
        name(a.name);
        put_be(h, uint64_t(a.type), 4);
        if (a.type == NC_CHAR) {
          put_be(h, a.text.size(), 4);
          h.insert(h.end(), a.text.begin(), a.text.end());
        } else {
          put_be(h, a.num.size(), 4);
          for (double x : a.num) encode(h, x, a.type);
        }
        while (h.size() % 4) h.push_back(0);
      }
    };
    if (dims_.empty()) { put_be(h, 0, 4); put_be(h, 0, 4); }
    else {
      put_be(h, TAG_DIMENSION, 4);
      put_be(h, dims_.size(), 4);
      for (const Dim& d : dims_) { name(d.name); put_be(h, d.len, 4); }
    }
    atts(gatts_);
    if (vs.empty()) { put_be(h, 0, 4); put_be(h, 0, 4); }
    else {
      put_be(h, TAG_VARIABLE, 4);
      put_be(h, vs.size(), 4);
      for (const Var& v : vs) {
        name(v.name);
        put_be(h, v.dims.size(), 4);
        for (int id : v.dims) put_be(h, uint64_t(id), 4);
        atts(v.atts);
        put_be(h, uint64_t(v.type), 4);
        put_be(h, v.vsize > 0xFFFFFFFFULL ? 0xFFFFFFFFULL : v.vsize, 4);
        put_be(h, v.begin, version == 2 ? 8 : 4);
      }
    }
    return h;
  };
  const uint64_t total_guess = fixed_total + recsize * numrecs_;
  const int version = total_guess > 0x7FFF0000ULL ? 2 : 1;
  const uint64_t hsize = header(version, vars).size();
  uint64_t off = hsize;
  for (Var& v : vars)
    if (!v.record) { v.begin = off; off += v.vsize; }
  for (Var& v : vars)
    if (v.record) { v.begin = off; off += v.vsize; }
  const std::vector<unsigned char> h = header(version, vars);
  FILE* fp = std::fopen(path.c_str(), "wb");
  if (!fp) { *err = "cannot create " + path; return false; }
  bool ok = std::fwrite(h.data(), 1, h.size(), fp) == h.size();
  const unsigned char zeros[4] = {0, 0, 0, 0};
  for (size_t i = 0; i < vars.size() && ok; ++i) {
    if (vars[i].record) continue;
    ok = std::fwrite(data_[i].data(), 1, data_[i].size(), fp) == data_[i].size();
    if (ok && vars[i].vsize > data_[i].size())
      ok = std::fwrite(zeros, 1, size_t(vars[i].vsize - data_[i].size()), fp) == vars[i].vsize - data_[i].size();
  }
  for (uint64_t r = 0; r < numrecs_ && ok; ++r)
    for (size_t i = 0; i < vars.size() && ok; ++i) {
      if (!vars[i].record) continue;
      const size_t slice = data_[i].size() / size_t(numrecs_);
      ok = std::fwrite(data_[i].data() + r * slice, 1, slice, fp) == slice;
      const uint64_t padded = nrec == 1 ? slice : vars[i].vsize;
      if (ok && padded > slice) ok = std::fwrite(zeros, 1, size_t(padded - slice), fp) == padded - slice;
    }
  if (std::fclose(fp) != 0 || !ok) { *err = "write failed: " + path; return false; }
  return true;
}

}  // namespace nc3
