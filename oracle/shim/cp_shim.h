// Minimal stand-ins for the absl and glog symbols that the reference CPU path
// (src/model/{types,intermediate_model,model_builder}.cpp, src/Network.cpp and
// the solver sources) uses. Test infrastructure only: it lets the oracle recipe
// compile the reference's own sources unmodified, because absl and glog are not
// installed in this image. Written for this project; behaviour follows the
// documented absl/glog semantics only as far as those sources rely on them.
#pragma once

#include <cctype>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <iostream>
#include <optional>
#include <sstream>
#include <string>
#include <string_view>
#include <type_traits>
#include <unordered_map>
#include <unordered_set>
#include <utility>
#include <vector>

namespace absl {

using string_view = std::string_view;

// ---- containers -----------------------------------------------------------
template <typename T, std::size_t N = 4>
using InlinedVector = std::vector<T>;

template <typename T>
class Span {
 public:
  Span() = default;
  Span(const T* p, std::size_t n) : p_(p), n_(n) {}
  template <typename C, typename = decltype(std::declval<const C&>().data())>
  Span(const C& c) : p_(c.data()), n_(c.size()) {}
  const T* begin() const { return p_; }
  const T* end() const { return p_ + n_; }
  const T* data() const { return p_; }
  std::size_t size() const { return n_; }
  bool empty() const { return n_ == 0; }
  const T& operator[](std::size_t i) const { return p_[i]; }

 private:
  const T* p_ = nullptr;
  std::size_t n_ = 0;
};

template <typename C>
auto MakeConstSpan(const C& c) {
  using T = std::remove_cv_t<std::remove_reference_t<decltype(*c.data())>>;
  return Span<const T>(c.data(), c.size());
}

// Hash state accepted by the reference's AbslHashValue overloads
// (H::combine(std::move(h), int)).
struct ShimHashState {
  std::size_t v = 0x9e3779b97f4a7c15ull;
  template <typename... Ts>
  static ShimHashState combine(ShimHashState h, const Ts&... xs) {
    ((h.v = (h.v ^ std::hash<Ts>{}(xs)) * 0x100000001b3ull), ...);
    return h;
  }
};

template <typename K, typename = void>
struct ShimHasher {
  std::size_t operator()(const K& k) const {
    return AbslHashValue(ShimHashState{}, k).v;
  }
};
template <typename K>
struct ShimHasher<K, std::void_t<decltype(std::hash<K>{}(std::declval<const K&>()))>> {
  std::size_t operator()(const K& k) const { return std::hash<K>{}(k); }
};
// String keys hash transparently, so lookups by string_view work as in absl.
template <>
struct ShimHasher<std::string, void> {
  using is_transparent = void;
  std::size_t operator()(std::string_view k) const { return std::hash<std::string_view>{}(k); }
};

template <typename K, typename V>
using flat_hash_map = std::unordered_map<K, V, ShimHasher<K>, std::equal_to<>>;
template <typename K>
using flat_hash_set = std::unordered_set<K, ShimHasher<K>, std::equal_to<>>;

// ---- strings --------------------------------------------------------------
namespace shim_detail {
inline void put(std::ostringstream& os, const std::string& s) { os << s; }
inline void put(std::ostringstream& os, std::string_view s) { os << s; }
inline void put(std::ostringstream& os, const char* s) { os << s; }
template <typename T>
void put(std::ostringstream& os, const T& v) { os << v; }

// Replace each printf conversion (%d, %s, %zu, %.2f, ...) with the next
// argument streamed in default format; "%%" prints a percent sign.
inline void fmt(std::ostringstream& os, const char* f) {
  for (; *f; ++f) {
    if (f[0] == '%' && f[1] == '%') { os << '%'; ++f; continue; }
    os << *f;
  }
}
template <typename A, typename... Rest>
void fmt(std::ostringstream& os, const char* f, const A& a, const Rest&... rest) {
  for (; *f; ++f) {
    if (f[0] == '%' && f[1] == '%') { os << '%'; ++f; continue; }
    if (f[0] == '%') {
      ++f;
      while (*f && !std::isalpha(static_cast<unsigned char>(*f))) ++f;
      while (*f == 'l' || *f == 'z' || *f == 'h') ++f;
      put(os, a);
      if (*f) ++f;
      fmt(os, f, rest...);
      return;
    }
    os << *f;
  }
}
}  // namespace shim_detail

template <typename... Args>
std::string StrFormat(const char* f, const Args&... args) {
  std::ostringstream os;
  shim_detail::fmt(os, f, args...);
  return os.str();
}

template <typename C>
std::string StrJoin(const C& parts, std::string_view sep) {
  std::ostringstream os;
  bool first = true;
  for (const auto& p : parts) {
    if (!first) os << sep;
    first = false;
    os << p;
  }
  return os.str();
}

template <typename... Args>
std::string StrCat(const Args&... args) {
  std::ostringstream os;
  (shim_detail::put(os, args), ...);
  return os.str();
}

// ---- status ---------------------------------------------------------------
class Status {
 public:
  Status() = default;
  explicit Status(std::string msg) : ok_(false), msg_(std::move(msg)) {}
  bool ok() const { return ok_; }
  const std::string& message() const { return msg_; }
  std::string ToString() const { return ok_ ? "OK" : msg_; }

 private:
  bool ok_ = true;
  std::string msg_;
};
inline Status OkStatus() { return Status(); }
inline Status InvalidArgumentError(std::string_view m) { return Status(std::string(m)); }

template <typename T>
class StatusOr {
 public:
  StatusOr(Status s) : status_(std::move(s)) {}
  StatusOr(T&& v) : value_(std::move(v)) {}
  bool ok() const { return value_.has_value(); }
  const Status& status() const { return status_; }
  T& value() & { return *value_; }
  const T& value() const& { return *value_; }
  T&& value() && { return std::move(*value_); }
  T& operator*() & { return *value_; }
  const T& operator*() const& { return *value_; }
  T* operator->() { return &*value_; }
  const T* operator->() const { return &*value_; }

 private:
  Status status_;
  std::optional<T> value_;
};

}  // namespace absl

// ---- glog -------------------------------------------------------------------
namespace shim_glog {
struct Sink {
  std::ostringstream os;
  bool fatal = false;
  bool quiet = false;
  ~Sink() {
    if (fatal) {
      std::cerr << "CHECK failed: " << os.str() << std::endl;
      std::abort();
    }
    if (!quiet && std::getenv("CP_SHIM_LOG")) std::cerr << os.str() << std::endl;
  }
  template <typename T>
  Sink& operator<<(const T& v) { os << v; return *this; }
};
struct Voidify {
  void operator&(Sink&) {}
};
}  // namespace shim_glog

#define CHECK(cond) \
  (cond) ? (void)0 : shim_glog::Voidify() & (shim_glog::Sink{{}, true, false} << #cond << " ")
#define CHECK_LE(a, b) CHECK((a) <= (b))
#define LOG(sev) shim_glog::Sink{}
