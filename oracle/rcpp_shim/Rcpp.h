// Test-only stand-in for the small part of the Rcpp API that fastEmbedR's CPU cores
// (src/tsne_neighbors.cpp, src/fast_knn_umap.cpp, src/embedding_utils.cpp) use, so that those
// files compile unchanged into the CPU reference library under oracle/_ref. R-level objects
// the bridge never reads (S4 payloads, R function calls, named list access) only compile.
// R is not needed: a SEXP here is a tagged, reference-counted numeric/integer vector or matrix
// (column-major).
// Written for this project; it shares only names and call signatures with Rcpp.
#ifndef FASTEMBEDR_TEST_RCPP_SHIM_H
#define FASTEMBEDR_TEST_RCPP_SHIM_H

#include <any>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstddef>
#include <cstdio>
#include <iostream>
#include <limits>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

typedef std::ptrdiff_t R_xlen_t;

enum { NILSXP = 0, LGLSXP = 10, INTSXP = 13, REALSXP = 14, STRSXP = 16, VECSXP = 19 };

struct SEXPREC : std::enable_shared_from_this<SEXPREC> {
  int type = NILSXP;
  std::vector<double> dbl;
  std::vector<int> ints;
  int nrow = -1;
  int ncol = -1;
};
typedef SEXPREC* SEXP;

static const int NA_INTEGER = INT_MIN;
static const double NA_REAL = std::numeric_limits<double>::quiet_NaN();
static const double R_NaReal = std::numeric_limits<double>::quiet_NaN();
static const double R_NaN = std::numeric_limits<double>::quiet_NaN();
static SEXPREC shim_dim_symbol_storage;
static const SEXP R_DimSymbol = &shim_dim_symbol_storage;
static const SEXP R_NilValue = nullptr;

inline int TYPEOF(SEXP x) { return x == nullptr ? NILSXP : x->type; }
inline bool Rf_isNull(SEXP x) { return x == nullptr || x->type == NILSXP; }
inline bool Rf_isS4(SEXP) { return false; }
inline bool Rf_isReal(SEXP x) { return x != nullptr && x->type == REALSXP; }
inline bool Rf_isMatrix(SEXP x) { return x != nullptr && x->nrow >= 0 && x->ncol >= 0; }
inline SEXP Rf_getAttrib(SEXP x, SEXP) { return Rf_isMatrix(x) ? x : nullptr; }
inline int* INTEGER(SEXP x) { return x->ints.data(); }
inline double* REAL(SEXP x) { return x->dbl.data(); }
inline R_xlen_t Rf_xlength(SEXP x) {
  if (x == nullptr) return 0;
  return static_cast<R_xlen_t>(x->type == REALSXP ? x->dbl.size() : x->ints.size());
}
inline int Rf_length(SEXP x) { return static_cast<int>(Rf_xlength(x)); }

namespace Rcpp {

inline std::string shim_format(const char* fmt, va_list ap) {
  char buf[2048];
  std::vsnprintf(buf, sizeof(buf), fmt, ap);
  return std::string(buf);
}

[[noreturn]] inline void stop(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  const std::string msg = shim_format(fmt, ap);
  va_end(ap);
  throw std::runtime_error(msg);
}
[[noreturn]] inline void stop(const std::string& msg) { throw std::runtime_error(msg); }

inline void warning(const char*, ...) {}
inline void warning(const std::string&) {}
inline void checkUserInterrupt() {}
static std::ostream& Rcout = std::cout;

struct NamedArg {
  std::string name;
  std::any value;
};

// Element of a create() call: a plain value, or the value of a Named(...) = value argument
// (names are not kept).
template <typename T, typename A>
T shim_item(const A& a) {
  return static_cast<T>(a);
}
template <typename T>
T shim_item(const NamedArg& a) {
  if (auto p = std::any_cast<double>(&a.value)) return static_cast<T>(*p);
  if (auto p = std::any_cast<int>(&a.value)) return static_cast<T>(*p);
  if (auto p = std::any_cast<float>(&a.value)) return static_cast<T>(*p);
  if (auto p = std::any_cast<bool>(&a.value)) return static_cast<T>(*p);
  throw std::runtime_error("shim: unsupported named element " + a.name);
}

// Stand-in for any R object the test bridge never reads (results of R calls, S4 slots, list
// elements by name): assignments are dropped and reading it throws.
struct ShimOpaque {
  template <typename T>
  ShimOpaque& operator=(const T&) {
    return *this;
  }
  template <typename T>
  operator T() const {
    throw std::runtime_error("shim: R objects are not available");
  }
};

template <int RTYPE, typename T>
class VectorBase {
 public:
  typedef T* iterator;
  typedef const T* const_iterator;

  VectorBase() : p_(std::make_shared<SEXPREC>()) { p_->type = RTYPE; }
  template <typename I, typename = typename std::enable_if<std::is_integral<I>::value>::type>
  VectorBase(I n) : VectorBase() { store().assign(static_cast<std::size_t>(n), T()); }
  template <typename I, typename = typename std::enable_if<std::is_integral<I>::value>::type>
  VectorBase(I n, const T& fill) : VectorBase() { store().assign(static_cast<std::size_t>(n), fill); }
  VectorBase(SEXP x) {
    if (x == nullptr || x->type != RTYPE) throw std::runtime_error("shim: SEXP type mismatch");
    p_ = x->shared_from_this();
  }
  template <typename It, typename = decltype(*std::declval<It>())>
  VectorBase(It first, It last) : VectorBase() {
    for (; first != last; ++first) store().push_back(static_cast<T>(*first));
  }
  template <typename... Args>
  static VectorBase create(Args... args) {
    VectorBase out;
    (out.store().push_back(shim_item<T>(args)), ...);
    return out;
  }
  operator SEXP() const { return p_.get(); }
  R_xlen_t size() const { return static_cast<R_xlen_t>(cstore().size()); }
  R_xlen_t length() const { return size(); }
  T& operator[](R_xlen_t i) { return store()[static_cast<std::size_t>(i)]; }
  const T& operator[](R_xlen_t i) const { return cstore()[static_cast<std::size_t>(i)]; }
  iterator begin() { return store().data(); }
  iterator end() { return store().data() + store().size(); }
  const_iterator begin() const { return cstore().data(); }
  const_iterator end() const { return cstore().data() + cstore().size(); }
  std::shared_ptr<SEXPREC> holder() const { return p_; }

 protected:
  std::vector<T>& store();
  const std::vector<T>& cstore() const;
  std::shared_ptr<SEXPREC> p_;
};

template <>
inline std::vector<double>& VectorBase<REALSXP, double>::store() { return p_->dbl; }
template <>
inline const std::vector<double>& VectorBase<REALSXP, double>::cstore() const { return p_->dbl; }
template <>
inline std::vector<int>& VectorBase<INTSXP, int>::store() { return p_->ints; }
template <>
inline const std::vector<int>& VectorBase<INTSXP, int>::cstore() const { return p_->ints; }

template <int RTYPE, typename T>
class MatrixBase : public VectorBase<RTYPE, T> {
 public:
  MatrixBase() : VectorBase<RTYPE, T>() { this->p_->nrow = 0; this->p_->ncol = 0; }
  MatrixBase(int nrow, int ncol)
      : VectorBase<RTYPE, T>(static_cast<R_xlen_t>(nrow) * static_cast<R_xlen_t>(ncol)) {
    this->p_->nrow = nrow;
    this->p_->ncol = ncol;
  }
  MatrixBase(SEXP x) : VectorBase<RTYPE, T>(x) {
    if (x->nrow < 0) throw std::runtime_error("shim: not a matrix");
  }
  int nrow() const { return this->p_->nrow; }
  int ncol() const { return this->p_->ncol; }
  T& operator()(int i, int j) {
    return this->store()[static_cast<std::size_t>(j) * static_cast<std::size_t>(nrow()) + static_cast<std::size_t>(i)];
  }
  const T& operator()(int i, int j) const {
    return this->cstore()[static_cast<std::size_t>(j) * static_cast<std::size_t>(nrow()) + static_cast<std::size_t>(i)];
  }
};

typedef VectorBase<REALSXP, double> NumericVector;
typedef VectorBase<INTSXP, int> IntegerVector;
typedef MatrixBase<REALSXP, double> NumericMatrix;
typedef MatrixBase<INTSXP, int> IntegerMatrix;

struct Named {
  explicit Named(const std::string& n) : name(n) {}
  template <typename T>
  NamedArg operator=(const T& v) const {
    return NamedArg{name, std::any(v)};
  }
  NamedArg operator=(const char* v) const { return NamedArg{name, std::any(std::string(v))}; }
  std::string name;
};

class List {
 public:
  template <typename... Args>
  static List create(Args... args) {
    List out;
    (out.items_.push_back(args), ...);
    return out;
  }
  bool has(const std::string& n) const {
    for (const auto& it : items_)
      if (it.name == n) return true;
    return false;
  }
  const std::any& get(const std::string& n) const {
    for (const auto& it : items_)
      if (it.name == n) return it.value;
    throw std::runtime_error("shim: list element not found: " + n);
  }
  ShimOpaque operator[](const char*) { return ShimOpaque(); }

 private:
  std::vector<NamedArg> items_;
};

class S4 {
 public:
  explicit S4(SEXP) {}
  explicit S4(const char*) {}
  bool is(const char*) const { return false; }
  ShimOpaque slot(const char*) const { return ShimOpaque(); }
  operator SEXP() const { throw std::runtime_error("shim: S4 objects are not available"); }
};

// R-level calls (base::qr, base::svd, ...) are not available; only their call syntax compiles.
class Function {
 public:
  Function() = default;
  template <typename... Args>
  ShimOpaque operator()(Args...) const {
    throw std::runtime_error("shim: R functions are not available");
  }
};

class Environment {
 public:
  static Environment base_env() { return Environment(); }
  Function operator[](const char*) const { return Function(); }
};

template <typename T, typename X>
T as(const X&) {
  throw std::runtime_error("shim: Rcpp::as is not available");
}

struct CharacterVector {
  template <typename... Args>
  static CharacterVector create(Args...) {
    return CharacterVector();
  }
};

template <typename M>
ShimOpaque colnames(M&) {
  return ShimOpaque();
}

inline IntegerVector wrap(const std::vector<int>& v) { return IntegerVector(v.begin(), v.end()); }
inline NumericVector wrap(const std::vector<float>& v) { return NumericVector(v.begin(), v.end()); }
inline NumericVector wrap(const std::vector<double>& v) { return NumericVector(v.begin(), v.end()); }

inline NumericMatrix clone(const NumericMatrix& m) {
  NumericMatrix out(m.nrow(), m.ncol());
  std::copy(m.begin(), m.end(), out.begin());
  return out;
}
inline IntegerMatrix clone(const IntegerMatrix& m) {
  IntegerMatrix out(m.nrow(), m.ncol());
  std::copy(m.begin(), m.end(), out.begin());
  return out;
}

}  // namespace Rcpp

#endif
