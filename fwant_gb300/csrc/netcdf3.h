// NetCDF classic-format files (CDF-1, and CDF-2 with 64-bit offsets): the on-disk format
// of every input and output file of the reference's solver (coord_, metric_, media_,
// source_, station_, seismo_, vel_/sgt_ snapshot files; nfseis_* in
// code/srcF/mod_nfseis.F90, written through the netCDF-Fortran library).  Written from the
// published format specification: a big-endian header of dimensions, attributes and
// variables, then the fixed-size variables, then the records of the variables along the
// unlimited dimension.  Dimensions are listed slowest first, so reading a variable's
// elements in file order yields the Fortran (first index fastest) order.
#pragma once
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

namespace nc3 {

enum Type { NC_BYTE = 1, NC_CHAR = 2, NC_SHORT = 3, NC_INT = 4, NC_FLOAT = 5, NC_DOUBLE = 6 };
int type_size(int type);

struct Dim {
  std::string name;
  uint64_t len = 0;  // 0 for the record (unlimited) dimension
};

struct Att {
  std::string name;
  int type = NC_CHAR;
  std::vector<double> num;  // numeric values
  std::string text;         // NC_CHAR values
};

struct Var {
  std::string name;
  std::vector<int> dims;    // dimension ids, slowest first
  std::vector<Att> atts;
  int type = NC_FLOAT;
  uint64_t vsize = 0;       // bytes of the variable (of one record for record variables)
  uint64_t begin = 0;       // file offset of the data (of the first record)
  bool record = false;
};

// Read-only view of a file (header parsed on open, data read on request).
class Reader {
 public:
  ~Reader();
  bool open(const std::string& path, std::string* err);
  const Dim* dim(const std::string& name) const;
  const Var* var(const std::string& name) const;
  const Att* gatt(const std::string& name) const;
  uint64_t numrecs() const { return numrecs_; }
  // number of elements of a variable (records included)
  uint64_t count(const Var& v) const;
  // whole variable converted to the requested element type, in file order
  bool read(const std::string& name, std::vector<double>* out, std::string* err) const;
  bool read(const std::string& name, std::vector<float>* out, std::string* err) const;
  bool read(const std::string& name, std::vector<int>* out, std::string* err) const;
  // strided hyperslab (per dimension, slowest first: 0-based start, count, stride >= 1; for
  // a record variable the first dimension counts records) converted to float, slab
  // elements in file order (last dimension fastest) -- nf90_get_var with start/count/stride
  bool read_slab(const std::string& name, const std::vector<uint64_t>& start, const std::vector<uint64_t>& count,
                 const std::vector<uint64_t>& stride, std::vector<float>* out, std::string* err) const;
  std::vector<Dim> dims;
  std::vector<Att> gatts;
  std::vector<Var> vars;

 private:
  bool read_raw(const Var& v, std::vector<double>* out, std::string* err) const;
  friend bool update_slab(const std::string&, const std::string&, const std::vector<uint64_t>&,
                          const std::vector<uint64_t>&, const std::vector<uint64_t>&, const float*, std::string*);
  FILE* fp_ = nullptr;
  uint64_t numrecs_ = 0, recsize_ = 0;
};

// Builds a file in memory and writes it in one go.
class Writer {
 public:
  int add_dim(const std::string& name, uint64_t len);  // len 0: the record dimension
  void add_gatt_text(const std::string& name, const std::string& text);
  void add_gatt(const std::string& name, int type, const std::vector<double>& values);
  // data: elements in file order (for a record variable all records, numrecs of them)
  int add_var(const std::string& name, int type, const std::vector<int>& dims, const std::vector<double>& data);
  int add_var_f(const std::string& name, const std::vector<int>& dims, const float* data, size_t n);
  int add_var_i(const std::string& name, const std::vector<int>& dims, const int* data, size_t n);
  int add_var_c(const std::string& name, const std::vector<int>& dims, const char* data, size_t n);
  void set_numrecs(uint64_t n) { numrecs_ = n; }
  bool write(const std::string& path, std::string* err) const;

 private:
  std::vector<Dim> dims_;
  std::vector<Att> gatts_;
  std::vector<Var> vars_;
  std::vector<std::vector<unsigned char>> data_;  // big-endian element bytes, file order
  uint64_t numrecs_ = 0;
};

// Writes a strided hyperslab of a fixed-size NC_FLOAT variable of an existing file in
// place (nf90_put_var with start/count/stride on a file opened for writing); data in slab
// file order.  The rest of the file is left as it is.
bool update_slab(const std::string& path, const std::string& name, const std::vector<uint64_t>& start,
                 const std::vector<uint64_t>& count, const std::vector<uint64_t>& stride, const float* data,
                 std::string* err);

}  // namespace nc3
