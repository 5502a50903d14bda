// Key/column configuration files (SeisFD3D.conf), read with the semantics of the
// reference's string_conf (code/srcF/mod_string.F90:166-282): on every line '#' starts a
// comment, the characters '=', tab and '|' separate words like blanks, and the value of
// (key, column c) is the c-th word of the first line whose first word is the key.
#pragma once
#include <cstddef>
#include <string>
#include <vector>

namespace conf {

class File {
 public:
  bool load(const std::string& path, std::string* err);
  bool has(const std::string& key) const;
  // the gcol-th word (1-based) of the line whose kcol-th word is key
  bool get(const std::string& key, int gcol, std::string* out, int kcol = 1) const;
  bool get_int(const std::string& key, int gcol, int* out) const;
  bool get_double(const std::string& key, int gcol, double* out) const;

 private:
  std::vector<std::vector<std::string>> lines_;
};

// A text input file read both ways the reference reads one: keys through string_conf, and
// the numbers after an anchor line (string_conf positions the unit after the line whose first
// word is the anchor) record by record, as Fortran list-directed reads take them: a record
// takes as many lines as its values need, commas separate values like blanks, and the rest of
// the record's last line is skipped.  Errors throw std::runtime_error naming the file.
class Text {
 public:
  explicit Text(const std::string& path);
  const std::string& path() const { return path_; }
  bool has(const std::string& key) const { return cf_.has(key); }
  int get_int(const std::string& key, int col) const;
  double get_double(const std::string& key, int col) const;
  std::string get(const std::string& key, int col) const;
  // position after the first line whose first word is the anchor
  void seek(const std::string& anchor);
  // one record of n words
  std::vector<std::string> words(size_t n);
  // one record of n single-precision values (each word rounded once to float)
  std::vector<float> record(size_t n);

 private:
  std::string path_;
  File cf_;
  std::vector<std::string> raw_;
  size_t line_ = 0;
};

// a word of a list-directed record as real(SP) or real(DP); throws on a non-number
float to_float(const std::string& word, const std::string& where);
double to_double(const std::string& word, const std::string& where);

}  // namespace conf
