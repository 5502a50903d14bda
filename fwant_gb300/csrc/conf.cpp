// Configuration-file reader (see conf.h).
#include "conf.h"

#include <cstdlib>
#include <fstream>
#include <sstream>
#include <stdexcept>

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

namespace {
std::string fortran_exponent(std::string s) {
  for (char& c : s)
    if (c == 'd' || c == 'D') c = 'e';
  return s;
}
}  // namespace

float to_float(const std::string& word, const std::string& where) {
  const std::string s = fortran_exponent(word);
  char* end = nullptr;
  const float f = std::strtof(s.c_str(), &end);
  if (end == s.c_str() || *end != '\0') throw std::runtime_error(where + ": not a number: " + word);
  return f;
}

double to_double(const std::string& word, const std::string& where) {
  const std::string s = fortran_exponent(word);
  char* end = nullptr;
  const double d = std::strtod(s.c_str(), &end);
  if (end == s.c_str() || *end != '\0') throw std::runtime_error(where + ": not a number: " + word);
  return d;
}

Text::Text(const std::string& path) : path_(path) {
  std::string err;
  if (!cf_.load(path, &err)) throw std::runtime_error(err);
  std::ifstream in(path);
  for (std::string l; std::getline(in, l);) raw_.push_back(l);
}

int Text::get_int(const std::string& key, int col) const {
  int v;
  if (!cf_.get_int(key, col, &v)) throw std::runtime_error(path_ + ": key " + key + " missing");
  return v;
}

double Text::get_double(const std::string& key, int col) const {
  double v;
  if (!cf_.get_double(key, col, &v)) throw std::runtime_error(path_ + ": key " + key + " missing");
  return v;
}

std::string Text::get(const std::string& key, int col) const {
  std::string v;
  if (!cf_.get(key, col, &v)) throw std::runtime_error(path_ + ": key " + key + " missing");
  return v;
}

void Text::seek(const std::string& anchor) {
  for (size_t q = 0; q < raw_.size(); ++q) {
    std::string l = raw_[q];
    const size_t h = l.find('#');
    if (h != std::string::npos) l.resize(h);
    for (char& c : l)
      if (c == '=' || c == '\t' || c == '|' || c == '\r') c = ' ';
    std::istringstream w(l);
    std::string first;
    if (w >> first && first == anchor) {
      line_ = q + 1;
      return;
    }
  }
  throw std::runtime_error(path_ + ": no " + anchor + " line");
}

std::vector<std::string> Text::words(size_t n) {
  std::vector<std::string> v;
  while (v.size() < n) {
    if (line_ >= raw_.size()) throw std::runtime_error(path_ + ": file ends inside a record");
    std::string l = raw_[line_++];
    for (char& c : l)
      if (c == ',' || c == '\t' || c == '\r') c = ' ';
    std::istringstream w(l);
    for (std::string t; v.size() < n && w >> t;) v.push_back(t);
  }
  return v;
}

std::vector<float> Text::record(size_t n) {
  std::vector<float> v;
  v.reserve(n);
  for (const std::string& t : words(n)) v.push_back(to_float(t, path_));
  return v;
}

}  // namespace conf
