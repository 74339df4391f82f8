// Minimal stand-in for boost::property_tree::ptree offering the get<T>(key,
// default) calls the solver set-up uses (TrilinosBelosSparseMatrixSolver.cpp
// :44-86).  Inside Phase the real Boost header is used.
#pragma once
#include <map>
#include <sstream>
#include <string>
namespace boost {
namespace property_tree {
class ptree {
 public:
  void put(const std::string &k, const std::string &v) { kv_[k] = v; }
  template <class T> T get(const std::string &k, const T &def) const {
    auto it = kv_.find(k);
    if (it == kv_.end()) return def;
    std::istringstream in(it->second);
    T v = def;
    in >> v;
    return v;
  }
 private:
  std::map<std::string, std::string> kv_;
};
}  // namespace property_tree
}  // namespace boost
