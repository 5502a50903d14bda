// Key/column configuration files (SeisFD3D.conf), read with the semantics of the
// reference's string_conf (code/srcF/mod_string.F90:166-282): on every line '#' starts a
// comment, the characters '=', tab and '|' separate words like blanks, and the value of
// (key, column c) is the c-th word of the first line whose first word is the key.
#pragma once
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

}  // namespace conf
