// Minimal no-op serialiser so that the reference's container headers compile
// without the Charm++ runtime; nothing here is ever called by the oracle.
#pragma once
#include <cstddef>
#include <string>
#include <vector>
#include <array>
#include <map>
#include <set>
#include <unordered_map>
#include <unordered_set>
#include <memory>
#include <functional>
#include <limits>
#include <cmath>
#include <algorithm>
#include <iostream>
#include <sstream>
#include <list>
#include <deque>
#include <tuple>
#include <utility>
#include <cstring>
#include <numeric>
#include <iomanip>
namespace PUP {
class er {
 public:
  virtual ~er() = default;
  bool isUnpacking() const { return false; }
  bool isPacking() const { return false; }
  bool isSizing() const { return false; }
  void operator()(char*, std::size_t) {}
  template <class T> void operator()(T&) {}
  template <class T> void operator()(T*, std::size_t) {}
};
template <class T> inline void operator|(er&, T&) {}
template <class T> inline void PUParray(er&, T*, std::size_t) {}
class able {};
using reconstruct = int;
}  // namespace PUP
