// Configuration-file reader (see conf.h).
#include "conf.h"

#include <cstdlib>
#include <fstream>
#include <sstream>

namespace conf {

bool File::load(const std::string& path, std::string* err) {
  std::ifstream in(path);
  if (!in) {
    *err = "cannot open " + path;
    return false;
  }
  std::string line;
  while (std::getline(in, line)) {
    const size_t hash = line.find('#');
    if (hash != std::string::npos) line.resize(hash);
    for (char& c : line)
      if (c == '=' || c == '\t' || c == '|' || c == '\r') c = ' ';
    std::istringstream words(line);
    std::vector<std::string> w;
    for (std::string s; words >> s;) w.push_back(s);
    if (!w.empty()) lines_.push_back(w);
  }
  return true;
}

bool File::get(const std::string& key, int gcol, std::string* out, int kcol) const {
  for (const auto& w : lines_) {
    if (int(w.size()) < kcol || w[kcol - 1] != key) continue;
    if (gcol < 1 || int(w.size()) < gcol) return false;
    *out = w[gcol - 1];
    return true;
  }
  return false;
}

bool File::has(const std::string& key) const {
  std::string s;
  return get(key, 1, &s);
}

bool File::get_int(const std::string& key, int gcol, int* out) const {
  std::string s;
  if (!get(key, gcol, &s)) return false;
  char* end = nullptr;
  const long v = std::strtol(s.c_str(), &end, 10);
  if (end == s.c_str() || *end != '\0') return false;
  *out = int(v);
  return true;
}

bool File::get_double(const std::string& key, int gcol, double* out) const {
  std::string s;
  if (!get(key, gcol, &s)) return false;
  for (char& c : s)
    if (c == 'd' || c == 'D') c = 'e';  // Fortran double-precision exponents
  char* end = nullptr;
  const double v = std::strtod(s.c_str(), &end);
  if (end == s.c_str() || *end != '\0') return false;
  *out = v;
  return true;
}

}  // namespace conf
