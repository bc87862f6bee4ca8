// lineal_gb300 C++ layer: GPU types that satisfy lineal's named requirements.
//
// lineal (KurtBoehm/lineal) is written against concepts, i.e. types are
// recognised by deriving from empty tag bases (include/lineal/base/concept/
// range.hpp:17-40, include/lineal/base/concept/solver.hpp:16-37) and by
// providing a set of members.  This header restates those tag bases and
// concepts and provides device-resident implementations whose bodies call the
// C ABI of include/lineal_gb300.h, so that code written in lineal's style --
// solver.instantiate(lhs, env), instance.instantiate(sol, rhs, env),
// system.iterate(env), run_iterative_solver(...) -- runs on a GB300.
//
// Header-only, C++20, no exceptions across the ABI: failures raise
// lineal::gb300::Error on the host side of this header.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <bit>
#include <cmath>
#include <concepts>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <optional>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#include "lineal_gb300.h"

namespace lineal::gb300 {

// ---- errors ------------------------------------------------------------------
struct Error : std::runtime_error {
  lgx_status status;
  Error(lgx_status s, const std::string &what) : std::runtime_error(what), status(s) {}
};

inline void check(lgx_status s) {
  if (s != LGX_OK)
    throw Error(s, std::string("lineal_gb300: ") + lgx_status_string(s) + ": " +
                     lgx_last_error());
}
inline void check_cuda(cudaError_t e) {
  if (e != cudaSuccess) throw Error(LGX_ERR_CUDA, cudaGetErrorString(e));
}

// ---- tag bases and concepts (base/concept/range.hpp:17-40, solver.hpp:16-37)
struct SharedVectorBase {};
struct SharedMatrixBase {};
struct SharedStationaryIterativeSolverBase {};
struct SharedNonStationaryIterativeSolverBase {};
struct SharedDirectSolverBase {};
struct EnvBase {};

template <typename T>
concept SharedVector = std::is_base_of_v<SharedVectorBase, std::decay_t<T>>;
template <typename T>
concept AnyVector = SharedVector<T>;
template <typename T>
concept SharedMatrix = std::is_base_of_v<SharedMatrixBase, std::decay_t<T>>;
template <typename T>
concept AnyMatrix = SharedMatrix<T>;
template <typename T>
concept StationaryIterativeSolver =
  std::is_base_of_v<SharedStationaryIterativeSolverBase, std::decay_t<T>>;
template <typename T>
concept NonStationaryIterativeSolver =
  std::is_base_of_v<SharedNonStationaryIterativeSolverBase, std::decay_t<T>>;
template <typename T>
concept DirectSolver = std::is_base_of_v<SharedDirectSolverBase, std::decay_t<T>>;
template <typename T>
concept Env = std::is_base_of_v<EnvBase, std::decay_t<T>>;

enum struct IsSymmetric : bool {};

// ---- environment (environment/environment.hpp:17-69) -------------------------
// The execution policy of a device environment is a CUDA stream.
struct DevicePolicy {
  cudaStream_t stream = nullptr;
  [[nodiscard]] std::size_t thread_num() const { return 1; }
};

struct Environment : EnvBase {
  explicit Environment(cudaStream_t s = nullptr) : policy_{s} {}
  [[nodiscard]] const DevicePolicy &execution_policy() const { return policy_; }
  [[nodiscard]] cudaStream_t stream() const { return policy_.stream; }
  template <typename T>
  void log(const char * /*name*/, const T & /*value*/) const {}
  [[nodiscard]] const Environment &add_object(const char * /*name*/ = nullptr) const {
    return *this;
  }
  [[nodiscard]] const Environment &dummy() const { return *this; }

 private:
  DevicePolicy policy_;
};

// ---- dense vectors (tensor/dynamic/dense/vector/shared.hpp:350-362) -----------
template <typename TValue = double>
class DenseVector : public SharedVectorBase {
 public:
  using Value = TValue;
  using Size = std::size_t;

  DenseVector() = default;
  explicit DenseVector(Size n) : n_(n) { alloc(); }
  DenseVector(Size n, const Environment & /*env*/) : DenseVector(n) {}
  DenseVector(Size n, Value value, const Environment &env) : DenseVector(n) {
    std::vector<Value> h(n, value);
    check_cuda(cudaMemcpyAsync(p_, h.data(), n * sizeof(Value), cudaMemcpyHostToDevice,
                               env.stream()));
    check_cuda(cudaStreamSynchronize(env.stream()));
  }
  DenseVector(const DenseVector &) = delete;
  DenseVector &operator=(const DenseVector &) = delete;
  DenseVector(DenseVector &&o) noexcept : n_(o.n_), p_(std::exchange(o.p_, nullptr)) {}
  DenseVector &operator=(DenseVector &&o) noexcept {
    std::swap(n_, o.n_);
    std::swap(p_, o.p_);
    return *this;
  }
  ~DenseVector() {
    if (p_) cudaFree(p_);
  }

  [[nodiscard]] Size size() const { return n_; }
  [[nodiscard]] Value *data() { return p_; }
  [[nodiscard]] const Value *data() const { return p_; }

  // Host element access (dense/vector/shared.hpp:268-310): the vector lives
  // in device memory, so every access is one synchronous copy of one
  // element -- for inspection and set-up, not for loops over the vector.
  // compute / store run on the environment's stream (after the work queued
  // there); operator[] uses a blocking copy, ordered after the legacy
  // default stream and every blocking stream.
  class ElementRef {
   public:
    ElementRef(DenseVector &v, Size i) : v_(v), i_(i) {}
    operator Value() const { return v_.read(i_); }  // NOLINT: a value proxy
    ElementRef &operator=(Value x) {
      v_.write(i_, x);
      return *this;
    }
    ElementRef &operator=(const ElementRef &o) { return *this = (Value)o; }

   private:
    DenseVector &v_;
    Size i_;
  };
  [[nodiscard]] Value operator[](Size i) const { return read(i); }
  [[nodiscard]] ElementRef operator[](Size i) { return ElementRef(*this, i); }
  [[nodiscard]] Value compute(Size i, const Environment &env) const {
    bounds(i);
    Value h{};
    check_cuda(cudaMemcpyAsync(&h, p_ + i, sizeof(Value), cudaMemcpyDeviceToHost, env.stream()));
    check_cuda(cudaStreamSynchronize(env.stream()));
    return h;
  }
  void store(Size i, Value v, const Environment &env) {
    bounds(i);
    check_cuda(cudaMemcpyAsync(p_ + i, &v, sizeof(Value), cudaMemcpyHostToDevice, env.stream()));
    check_cuda(cudaStreamSynchronize(env.stream()));
  }

  void upload(const std::vector<Value> &h, const Environment &env) {
    check_cuda(cudaMemcpyAsync(p_, h.data(), n_ * sizeof(Value), cudaMemcpyHostToDevice,
                               env.stream()));
    check_cuda(cudaStreamSynchronize(env.stream()));
  }
  [[nodiscard]] std::vector<Value> download(const Environment &env) const {
    std::vector<Value> h(n_);
    check_cuda(cudaMemcpyAsync(h.data(), p_, n_ * sizeof(Value), cudaMemcpyDeviceToHost,
                               env.stream()));
    check_cuda(cudaStreamSynchronize(env.stream()));
    return h;
  }

 private:
  void alloc() {
    if (n_) check_cuda(cudaMalloc(&p_, n_ * sizeof(Value)));
  }
  void bounds(Size i) const {
    if (i >= n_) throw std::out_of_range("DenseVector element index out of range");
  }
  [[nodiscard]] Value read(Size i) const {
    bounds(i);
    Value h{};
    check_cuda(cudaMemcpy(&h, p_ + i, sizeof(Value), cudaMemcpyDeviceToHost));
    return h;
  }
  void write(Size i, Value v) {
    bounds(i);
    check_cuda(cudaMemcpy(p_ + i, &v, sizeof(Value), cudaMemcpyHostToDevice));
  }
  Size n_ = 0;
  Value *p_ = nullptr;
};

template <typename TVec>
TVec create_numa_undef_like(const AnyMatrix auto &m, const Environment &env) {
  return TVec(m.row_num(), env);
}

// ---- matrices ---------------------------------------------------------------------
class MatrixHandle : public SharedMatrixBase {
 public:
  using Value = double;
  using Size = std::size_t;

  MatrixHandle() = default;
  explicit MatrixHandle(lgx_matrix *h) : h_(h) {}
  MatrixHandle(const MatrixHandle &) = delete;
  MatrixHandle &operator=(const MatrixHandle &) = delete;
  MatrixHandle(MatrixHandle &&o) noexcept : h_(std::exchange(o.h_, nullptr)) {}
  MatrixHandle &operator=(MatrixHandle &&o) noexcept {
    std::swap(h_, o.h_);
    return *this;
  }
  ~MatrixHandle() {
    if (h_) lgx_matrix_destroy(h_);
  }

  [[nodiscard]] lgx_matrix *handle() const { return h_; }
  [[nodiscard]] Size row_num() const { return (Size)info().n; }
  [[nodiscard]] Size column_num() const { return row_num(); }
  [[nodiscard]] Size non_zero_num() const { return (Size)info().nnz; }
  [[nodiscard]] IsSymmetric is_symmetric() const { return IsSymmetric{info().sym != 0}; }

 private:
  struct Info {
    int kind;
    int64_t n, nnz;
    int sym;
  };
  [[nodiscard]] Info info() const {
    Info i{};
    check(lgx_matrix_info(h_, &i.kind, &i.n, &i.nnz, &i.sym));
    return i;
  }
  lgx_matrix *h_ = nullptr;
};

// CsrMatrix (tensor/dynamic/csr/shared.hpp:1114-1116); built from host CSR
// arrays (RowWiseBuilder-style input: sorted columns, stored diagonal).
class CsrMatrix : public MatrixHandle {
 public:
  using MatrixHandle::MatrixHandle;
  static CsrMatrix from_host(const std::vector<int64_t> &rowptr, const std::vector<int32_t> &col,
                             const std::vector<double> &val, IsSymmetric sym,
                             lgx_dtype storage = LGX_F64) {
    lgx_matrix *h = nullptr;
    check(lgx_csr_create_host((int64_t)rowptr.size() - 1, (int64_t)col.size(), rowptr.data(),
                              col.data(), val.data(), sym == IsSymmetric{true}, storage, &h));
    return CsrMatrix(h);
  }
  // the synthetic 27-point lognormal operator on a grid (device generator)
  static CsrMatrix diffusion_27pt(const int64_t dims[3], const DenseVector<double> &k,
                                  const Environment &env, lgx_dtype storage = LGX_F64) {
    lgx_matrix *h = nullptr;
    check(lgx_gen_27pt(dims, k.data(), storage, env.stream(), &h));
    return CsrMatrix(h);
  }
};

// Host row access to a CSR matrix (csr/shared.hpp:120-333, 926-1036): one
// download of the whole matrix (rows, sorted columns, values), then rows with
// lineal's ConstRow interface -- size, index, column indices, find /
// contains, value by column, iterate over all entries or split around the
// diagonal.  The matrix stays in device memory; the snapshot does not follow
// later changes.  An iterate operation that returns a std::optional ends the
// walk at the first engaged value and returns it (lineal's valued returns).
class HostCsr {
 public:
  using Size = std::size_t;
  using Value = double;
  using ColumnIdx = int32_t;

  class ConstRow {
   public:
    ConstRow(const int32_t *col, const double *val, Size row, Size nnz)
        : col_(col), val_(val), row_(row), nnz_(nnz) {}
    [[nodiscard]] Size index() const { return row_; }
    [[nodiscard]] Size size() const { return nnz_; }
    [[nodiscard]] Size offdiagonal_num() const { return contains((ColumnIdx)row_) ? nnz_ - 1 : nnz_; }
    [[nodiscard]] std::vector<ColumnIdx> column_indices() const {
      return std::vector<ColumnIdx>(col_, col_ + nnz_);
    }
    // position of column c among the row's entries, or none
    [[nodiscard]] std::optional<Size> find(ColumnIdx c) const {
      const int32_t *it = std::lower_bound(col_, col_ + nnz_, c);
      if (it == col_ + nnz_ || *it != c) return std::nullopt;
      return (Size)(it - col_);
    }
    [[nodiscard]] bool contains(ColumnIdx c) const { return find(c).has_value(); }
    // the entry in column c (an absent column is an error: lineal asserts)
    [[nodiscard]] Value operator[](ColumnIdx c) const {
      const auto k = find(c);
      if (!k) throw std::out_of_range("HostCsr row has no entry in this column");
      return val_[*k];
    }
    // the diagonal entry (lineal's rows always store it)
    [[nodiscard]] Value diagonal() const { return (*this)[(ColumnIdx)row_]; }
    // position of column c among the row's off-diagonal entries
    [[nodiscard]] Size offdiagonal_index_within(ColumnIdx c) const {
      const auto k = find(c);
      if (!k || (Size)c == row_) throw std::out_of_range("no off-diagonal entry in this column");
      return *k - ((Size)c > row_ && contains((ColumnIdx)row_) ? 1 : 0);
    }
    [[nodiscard]] Value back() const { return val_[nnz_ - 1]; }
    [[nodiscard]] ColumnIdx back_column() const { return col_[nnz_ - 1]; }
    // op(column, value) for every entry in column order
    template <typename Op>
    auto iterate(Op op) const {
      using Ret = decltype(op(ColumnIdx{}, Value{}));
      for (Size k = 0; k < nnz_; ++k) {
        if constexpr (is_optional<Ret>) {
          if (auto r = op(col_[k], val_[k])) return r;
        } else {
          op(col_[k], val_[k]);
        }
      }
      if constexpr (is_optional<Ret>) return Ret{};
    }
    // before(column, value) for the columns left of the diagonal,
    // diagonal(column, value) for the diagonal, after(...) for the rest
    template <typename B, typename D, typename A>
    void iterate(B before, D diagonal, A after) const {
      for (Size k = 0; k < nnz_; ++k) {
        const ColumnIdx c = col_[k];
        if ((Size)c < row_) before(c, val_[k]);
        else if ((Size)c == row_) diagonal(c, val_[k]);
        else after(c, val_[k]);
      }
    }

   private:
    template <typename T>
    struct optional_check : std::false_type {};
    template <typename T>
    struct optional_check<std::optional<T>> : std::true_type {};
    template <typename T>
    static constexpr bool is_optional = optional_check<T>::value;

    const int32_t *col_;
    const double *val_;
    Size row_, nnz_;
  };

  static HostCsr download(const CsrMatrix &m, const Environment &env) {
    HostCsr h;
    const Size n = m.row_num(), nnz = m.non_zero_num();
    h.rowptr_.resize(n + 1);
    h.col_.resize(nnz);
    h.val_.resize(nnz);
    check(lgx_csr_download(m.handle(), h.rowptr_.data(), h.col_.data(), h.val_.data(),
                           env.stream()));
    return h;
  }
  [[nodiscard]] Size row_num() const { return rowptr_.empty() ? 0 : rowptr_.size() - 1; }
  [[nodiscard]] Size column_num() const { return row_num(); }
  [[nodiscard]] Size non_zero_num() const { return col_.size(); }
  [[nodiscard]] Value diagonal_at(Size row) const { return (*this)[row].diagonal(); }
  [[nodiscard]] Value entry_at(Size row, ColumnIdx c) const { return (*this)[row][c]; }
  // the CSR arrays themselves (csr/shared.hpp row_offsets / column_indices /
  // entries)
  [[nodiscard]] const std::vector<int64_t> &row_offsets() const { return rowptr_; }
  [[nodiscard]] const std::vector<int32_t> &column_indices() const { return col_; }
  [[nodiscard]] const std::vector<double> &entries() const { return val_; }
  [[nodiscard]] ConstRow operator[](Size row) const {
    if (row >= row_num()) throw std::out_of_range("HostCsr row index out of range");
    const int64_t b = rowptr_[row];
    return ConstRow(col_.data() + b, val_.data() + b, row, (Size)(rowptr_[row + 1] - b));
  }

 private:
  std::vector<int64_t> rowptr_;
  std::vector<int32_t> col_;
  std::vector<double> val_;
};

// BoxInfo (discretization/box-equidistant.hpp:57-110): cell counts and axis
// lengths of an equidistant box and the axis quotients the valuators use
struct BoxInfo {
  std::array<int64_t, 3> cell_nums;
  std::array<double, 3> lengths;

  BoxInfo(std::array<int64_t, 3> cells, std::array<double, 3> axis_lengths)
      : cell_nums(cells), lengths(axis_lengths) {
    (void)axis_quotients();  // validates
  }
  [[nodiscard]] std::array<double, 3> axis_lengths() const { return lengths; }
  [[nodiscard]] double axis_length(std::size_t axis) const { return lengths[axis]; }
  [[nodiscard]] std::array<double, 3> axis_quotients() const {
    lgx_box_info b{};
    for (int d = 0; d < 3; ++d) {
      b.cells[d] = cell_nums[d];
      b.lengths[d] = lengths[d];
    }
    std::array<double, 3> q{};
    check(lgx_box_axis_quotients(&b, q.data()));
    return q;
  }
  [[nodiscard]] double axis_quotient(std::size_t axis) const { return axis_quotients()[axis]; }
};

// AdjacentStencilMatrix with a StationaryDiffusionLookupValuator / ValueValuator
class StencilMatrix : public MatrixHandle {
 public:
  using MatrixHandle::MatrixHandle;
  // the valuators' BoxInfo constructors (stationary-diffusion-lookup.hpp:28-60)
  static StencilMatrix lookup(const BoxInfo &box, const double coeffs[4],
                              const DenseVector<uint8_t> &materials, double sol_start,
                              double sol_end, bool zero_to_one, const Environment &env) {
    const auto q = box.axis_quotients();
    return lookup(box.cell_nums.data(), q.data(), coeffs, materials, sol_start, sol_end,
                  zero_to_one, env);
  }
  static StencilMatrix value(const BoxInfo &box, const DenseVector<double> &k, double sol_start,
                             double sol_end, bool zero_to_one, const Environment &env) {
    const auto q = box.axis_quotients();
    return value(box.cell_nums.data(), q.data(), k, sol_start, sol_end, zero_to_one, env);
  }
  static StencilMatrix lookup(const int64_t dims[3], const double q[3], const double coeffs[4],
                              const DenseVector<uint8_t> &materials, double sol_start,
                              double sol_end, bool zero_to_one, const Environment &env) {
    lgx_matrix *h = nullptr;
    check(lgx_stencil_create_lookup(dims, q, coeffs, materials.data(), sol_start, sol_end,
                                    zero_to_one, env.stream(), &h));
    return StencilMatrix(h);
  }
  static StencilMatrix value(const int64_t dims[3], const double q[3],
                             const DenseVector<double> &k, double sol_start, double sol_end,
                             bool zero_to_one, const Environment &env) {
    lgx_matrix *h = nullptr;
    check(lgx_stencil_create_value(dims, q, k.data(), sol_start, sol_end, zero_to_one,
                                   env.stream(), &h));
    return StencilMatrix(h);
  }
  // StationaryDiffusionValuesValuator: one conductivity array per axis
  static StencilMatrix values(const int64_t dims[3], const double q[3],
                              const DenseVector<double> &k0, const DenseVector<double> &k1,
                              const DenseVector<double> &k2, double sol_start, double sol_end,
                              bool zero_to_one, const Environment &env) {
    lgx_matrix *h = nullptr;
    check(lgx_stencil_create_values(dims, q, k0.data(), k1.data(), k2.data(), sol_start, sol_end,
                                    zero_to_one, env.stream(), &h));
    return StencilMatrix(h);
  }
  // lookup valuator with HenryDiffusionLookupWright's diffusion factors
  static StencilMatrix lookup_henry(const int64_t dims[3], const double q[3],
                                    const double coeffs[4], uint8_t gaseous_materials,
                                    double henry_constant, const DenseVector<uint8_t> &materials,
                                    double sol_start, double sol_end, bool zero_to_one,
                                    const Environment &env) {
    lgx_matrix *h = nullptr;
    check(lgx_stencil_create_lookup_henry(dims, q, coeffs, gaseous_materials, henry_constant,
                                          materials.data(), sol_start, sol_end, zero_to_one,
                                          env.stream(), &h));
    return StencilMatrix(h);
  }
};

// EffDiffCalc (component-wise/sink/effective-diffusion.hpp:226-320): the
// effective diffusivity of a solution through the middle planes of axis 0.
// Constructed from the stencil (its axis lengths and "none" materials);
// the call takes the solution (and the compress map of a compressed system).
class EffDiffCalc {
 public:
  EffDiffCalc(const StencilMatrix &valuator, const std::array<double, 3> &axis_lengths,
              uint8_t none_materials = 0)
      : lengths_(axis_lengths), none_(none_materials) {
    (void)valuator;
  }
  double operator()(const StencilMatrix &valuator, const DenseVector<double> &sol,
                    const Environment &env) const {
    return (*this)(valuator, nullptr, sol, env);
  }
  double operator()(const StencilMatrix &valuator, const DenseVector<int64_t> *compress_map,
                    const DenseVector<double> &sol, const Environment &env) const {
    double eff = 0.0, area = 0.0;
    check(lgx_stencil_effective_diffusion(valuator.handle(), lengths_.data(), none_,
                                          sol.data(), compress_map ? compress_map->data() : nullptr,
                                          env.stream(), &eff, &area));
    return eff;
  }

 private:
  std::array<double, 3> lengths_;
  uint8_t none_;
};

// ---- component-wise operations (component-wise/*) ------------------------------
template <typename TLhs, typename TRhs>
struct MatrixVectorProductExpr {
  const TLhs &lhs;
  const TRhs &rhs;
};

template <AnyMatrix TLhs, AnyVector TRhs>
MatrixVectorProductExpr<TLhs, TRhs> operator*(const TLhs &lhs, const TRhs &rhs) {
  return {lhs, rhs};
}

// assign(y, A * x) (sink/assignment.hpp:114-117)
template <typename TLhs, typename TRhs>
void assign(DenseVector<double> &y, const MatrixVectorProductExpr<TLhs, TRhs> &e,
            const DevicePolicy &pol) {
  check(lgx_spmv(e.lhs.handle(), e.rhs.data(), y.data(), pol.stream));
}

// add / subtract / scale and operator+ - * (component-wise/vector-expression.hpp:
// 67-91, 150-167): a vector, a scaled vector, or the sum or difference of two
// of them, assigned in one pass with lineal's rounding (each product and the
// sum rounded once, lgx_lincomb); constant / constant_like (140-147) assign a
// value.  Deeper trees (a scaled sum, three terms) are not expressions here.
struct ScaledVector {
  double scalar;
  const DenseVector<double> *vec;
};
struct LinCombExpr {
  double alpha;
  const DenseVector<double> *x;
  double beta;
  const DenseVector<double> *y;
};
struct ConstantExpr {
  std::size_t size;
  double value;
};

template <typename T>
concept LinTerm = std::same_as<std::decay_t<T>, DenseVector<double>> ||
                  std::same_as<std::decay_t<T>, ScaledVector>;

namespace detail {
inline ScaledVector term(const DenseVector<double> &v) { return {1.0, &v}; }
inline ScaledVector term(const ScaledVector &t) { return t; }
}  // namespace detail

inline ScaledVector scale(const DenseVector<double> &v, double scalar) { return {scalar, &v}; }
inline ScaledVector operator*(const DenseVector<double> &v, double scalar) { return {scalar, &v}; }
inline ScaledVector operator*(double scalar, const DenseVector<double> &v) { return {scalar, &v}; }
template <LinTerm A, LinTerm B>
LinCombExpr add(const A &a, const B &b) {
  const ScaledVector ta = detail::term(a), tb = detail::term(b);
  return {ta.scalar, ta.vec, tb.scalar, tb.vec};
}
template <LinTerm A, LinTerm B>
LinCombExpr subtract(const A &a, const B &b) {
  const ScaledVector ta = detail::term(a), tb = detail::term(b);
  return {ta.scalar, ta.vec, -tb.scalar, tb.vec};
}
template <LinTerm A, LinTerm B>
LinCombExpr operator+(const A &a, const B &b) {
  return add(a, b);
}
template <LinTerm A, LinTerm B>
LinCombExpr operator-(const A &a, const B &b) {
  return subtract(a, b);
}
inline ConstantExpr constant(std::size_t size, double value) { return {size, value}; }
inline ConstantExpr constant_like(const DenseVector<double> &v, double value) {
  return {v.size(), value};
}

namespace detail {
inline void same_size(std::size_t a, std::size_t b) {
  if (a != b) throw Error(LGX_ERR_INVALID, "lineal_gb300: vector sizes differ");
}
}  // namespace detail

inline void assign(DenseVector<double> &out, const LinCombExpr &e, const DevicePolicy &pol) {
  detail::same_size(out.size(), e.x->size());
  detail::same_size(out.size(), e.y->size());
  check(lgx_lincomb((int64_t)out.size(), e.alpha, e.x->data(), e.beta, e.y->data(), out.data(),
                    pol.stream));
}
inline void assign(DenseVector<double> &out, const ScaledVector &e, const DevicePolicy &pol) {
  detail::same_size(out.size(), e.vec->size());
  check(lgx_lincomb((int64_t)out.size(), e.scalar, e.vec->data(), 0.0, nullptr, out.data(),
                    pol.stream));
}
inline void assign(DenseVector<double> &out, const ConstantExpr &e, const DevicePolicy &pol) {
  detail::same_size(out.size(), e.size);
  check(lgx_fill((int64_t)out.size(), e.value, out.data(), pol.stream));
}

// swap (sink/swap.hpp:31-123): the contents change places (here the storage)
inline void swap(DenseVector<double> &a, DenseVector<double> &b, const DevicePolicy & /*pol*/) {
  detail::same_size(a.size(), b.size());
  std::swap(a, b);
}

inline double scalar_from_device(const double *d, cudaStream_t s) {
  double h = 0.0;
  check_cuda(cudaMemcpyAsync(&h, d, sizeof(double), cudaMemcpyDeviceToHost, s));
  check_cuda(cudaStreamSynchronize(s));
  return h;
}

// dot / euclidean_squared / euclidean_norm / max_norm (sink/accumulator.hpp:151-218)
template <typename TReal = double>
TReal dot(const DenseVector<double> &a, const DenseVector<double> &b, const DevicePolicy &pol) {
  DenseVector<double> out(1);
  check(lgx_dot((int64_t)a.size(), a.data(), b.data(), out.data(), pol.stream));
  return scalar_from_device(out.data(), pol.stream);
}
template <typename TReal = double>
TReal euclidean_squared(const DenseVector<double> &a, const DevicePolicy &pol) {
  return dot<TReal>(a, a, pol);
}
template <typename TReal = double>
TReal euclidean_norm(const DenseVector<double> &a, const DevicePolicy &pol) {
  return std::sqrt(euclidean_squared<TReal>(a, pol));
}
template <typename TReal = double>
TReal max_norm(const DenseVector<double> &a, const DevicePolicy &pol) {
  DenseVector<double> out(1);
  check(lgx_max_norm((int64_t)a.size(), a.data(), out.data(), pol.stream));
  return scalar_from_device(out.data(), pol.stream);
}

// multiconsume with dot / euclidean_squared / euclidean_norm / max_norm
// consumers (sink/accumulator.hpp:126-218): the consumers name the vectors
// they read by position; each consumer is one deterministic reduction
// (lineal fuses them into one pass; the values are the same reductions)
template <typename TReal, std::size_t tI, std::size_t tJ>
struct DotConsumer {};
template <typename TReal, std::size_t tI>
struct EuclideanSquaredConsumer {};
template <typename TReal, std::size_t tI>
struct EuclideanNormConsumer {};
template <typename TReal, std::size_t tI>
struct MaxNormConsumer {};
template <typename TReal, std::size_t tI, std::size_t tJ>
constexpr DotConsumer<TReal, tI, tJ> dot_consumer() {
  return {};
}
template <typename TReal, std::size_t tI>
constexpr EuclideanSquaredConsumer<TReal, tI> euclidean_squared_consumer() {
  return {};
}
template <typename TReal, std::size_t tI>
constexpr EuclideanNormConsumer<TReal, tI> euclidean_norm_consumer() {
  return {};
}
template <typename TReal, std::size_t tI>
constexpr MaxNormConsumer<TReal, tI> max_norm_consumer() {
  return {};
}

namespace detail {
template <typename TReal, std::size_t tI, std::size_t tJ, typename TVecs>
TReal consume(DotConsumer<TReal, tI, tJ>, const TVecs &v, const DevicePolicy &pol) {
  return dot<TReal>(std::get<tI>(v), std::get<tJ>(v), pol);
}
template <typename TReal, std::size_t tI, typename TVecs>
TReal consume(EuclideanSquaredConsumer<TReal, tI>, const TVecs &v, const DevicePolicy &pol) {
  return euclidean_squared<TReal>(std::get<tI>(v), pol);
}
template <typename TReal, std::size_t tI, typename TVecs>
TReal consume(EuclideanNormConsumer<TReal, tI>, const TVecs &v, const DevicePolicy &pol) {
  return euclidean_norm<TReal>(std::get<tI>(v), pol);
}
template <typename TReal, std::size_t tI, typename TVecs>
TReal consume(MaxNormConsumer<TReal, tI>, const TVecs &v, const DevicePolicy &pol) {
  return max_norm<TReal>(std::get<tI>(v), pol);
}
}  // namespace detail

template <typename... TConsumers, typename... TVecs>
auto multiconsume(std::tuple<TConsumers...> consumers, std::tuple<TVecs...> vecs,
                  const DevicePolicy &pol) {
  return std::apply(
    [&](auto... c) { return std::tuple{detail::consume(c, vecs, pol)...}; }, consumers);
}

// ---- stationary solvers (iterative-stationary/*) --------------------------------
struct forward_tag_t {};
struct backward_tag_t {};
inline constexpr forward_tag_t forward_tag{};
inline constexpr backward_tag_t backward_tag{};
enum struct SorVariant : uint8_t { regular, ultra };

// JacobiSolver (jacobi/solver.hpp:38-39), one sweep per apply
struct JacobiSolver : SharedStationaryIterativeSolverBase {
  double relax = 1.0;
  explicit JacobiSolver(double r) : relax(r) {}
  template <AnyMatrix TLhs>
  struct Instance {
    const TLhs &lhs;
    double relax;
    static constexpr std::size_t in_situ_aux_size = 1;
    static constexpr std::size_t ex_situ_aux_size = 0;
    // ex situ: out = sweep(in)
    void apply(const DenseVector<double> *in, DenseVector<double> &out,
               const DenseVector<double> &rhs, const Environment &env) const {
      check(lgx_jacobi_sweep(lhs.handle(), relax, in ? in->data() : nullptr, out.data(),
                             rhs.data(), env.stream()));
    }
    // lineal's call shapes (SingleSweepImpl, broom.hpp:36-51): ex situ with
    // an aux tuple, and in situ, where sol moves to aux[0] and the sweep
    // writes sol
    template <typename TAux>
    void apply(const DenseVector<double> &in, DenseVector<double> &out,
               const DenseVector<double> &rhs, TAux && /*aux*/, const Environment &env) const {
      apply(&in, out, rhs, env);
    }
    template <typename TAux>
    void apply(DenseVector<double> &sol, const DenseVector<double> &rhs, TAux &&aux,
               const Environment &env) const {
      DenseVector<double> &tmp = std::get<0>(aux);
      swap(sol, tmp, env.execution_policy());
      apply(&tmp, sol, rhs, env);
    }
  };
  template <AnyMatrix TLhs>
  Instance<TLhs> instantiate(const TLhs &lhs, const Environment & /*env*/) const {
    return {lhs, relax};
  }
};

// Multicolour SorSolver / SsorSolver (gauss-seidel-variant/solver.hpp:91-96)
class Colouring {
 public:
  Colouring() = default;
  Colouring(const CsrMatrix &a, uint64_t seed, const Environment &env) {
    check(lgx_colouring_create_jp(a.handle(), seed, env.stream(), &h_));
  }
  Colouring(const Colouring &) = delete;
  Colouring &operator=(const Colouring &) = delete;
  Colouring(Colouring &&o) noexcept : h_(std::exchange(o.h_, nullptr)) {}
  ~Colouring() {
    if (h_) lgx_colouring_destroy(h_);
  }
  [[nodiscard]] lgx_colouring *handle() const { return h_; }

 private:
  lgx_colouring *h_ = nullptr;
};

template <typename TDir, SorVariant tVariant = SorVariant::regular>
struct SorSolver : SharedStationaryIterativeSolverBase {
  double relax = 1.0;
  explicit SorSolver(double r) : relax(r) {}
  struct Instance {
    const CsrMatrix &lhs;
    Colouring colouring;
    double relax;
    static constexpr std::size_t in_situ_aux_size = 1;
    static constexpr std::size_t ex_situ_aux_size = 0;
    void apply(const DenseVector<double> *in, DenseVector<double> &out,
               const DenseVector<double> &rhs, const Environment &env) const {
      check(lgx_sor_sweep(lhs.handle(), colouring.handle(), relax,
                          std::is_same_v<TDir, forward_tag_t>, tVariant == SorVariant::ultra,
                          in ? in->data() : nullptr, out.data(), rhs.data(), env.stream()));
    }
    // in situ (SingleSweepImpl, broom.hpp:43-51)
    void apply(DenseVector<double> &sol, const DenseVector<double> &rhs,
               const Environment &env) const {
      apply(&sol, sol, rhs, env);
    }
    // lineal's call shapes with an aux tuple (broom.hpp:36-51); in situ, sol
    // moves to aux[0] and the sweep writes sol (the multicolour sweep gives
    // the same bits in place)
    template <typename TAux>
    void apply(const DenseVector<double> &in, DenseVector<double> &out,
               const DenseVector<double> &rhs, TAux && /*aux*/, const Environment &env) const {
      apply(&in, out, rhs, env);
    }
    template <typename TAux>
    void apply(DenseVector<double> &sol, const DenseVector<double> &rhs, TAux &&aux,
               const Environment &env) const {
      DenseVector<double> &tmp = std::get<0>(aux);
      swap(sol, tmp, env.execution_policy());
      apply(&tmp, sol, rhs, env);
    }
  };
  Instance instantiate(const CsrMatrix &lhs, const Environment &env) const {
    return Instance{lhs, Colouring(lhs, 0x5eed, env), relax};
  }
};

// ---- direct solvers (direct/cholesky/solver.hpp:22-67, direct/lu/solver.hpp:21-66)
// The dense FP64 solve of the AMG's coarsest level on its own: the inverse is
// formed once by instantiate, each solve is one dense product.  CholeskySolver
// requires positive pivots (symmetric positive definite matrices), LuSolver
// nonzero ones (no pivoting, as lineal's LU).
template <int tKind>
struct DenseDirectSolver : SharedDirectSolverBase {
  class Instance {
   public:
    static constexpr std::size_t aux_size = 0;
    Instance(const CsrMatrix &lhs, const Environment &env) : lhs_(&lhs) {
      check(lgx_direct_create(lhs.handle(), tKind, env.stream(), &h_));
    }
    Instance(const Instance &) = delete;
    Instance &operator=(const Instance &) = delete;
    Instance(Instance &&o) noexcept : lhs_(o.lhs_), h_(std::exchange(o.h_, nullptr)) {}
    ~Instance() {
      if (h_) lgx_direct_destroy(h_);
    }
    // sol = lhs^-1 rhs (aux unused: the inverse needs no work vector)
    template <typename TAux>
    void solve(DenseVector<double> &sol, const DenseVector<double> &rhs, TAux && /*aux*/,
               const Environment &env) const {
      check(lgx_direct_solve(h_, rhs.data(), sol.data(), env.stream()));
    }
    void solve(DenseVector<double> &sol, const DenseVector<double> &rhs,
               const Environment &env) const {
      check(lgx_direct_solve(h_, rhs.data(), sol.data(), env.stream()));
    }
    [[nodiscard]] const CsrMatrix &lhs() const { return *lhs_; }

   private:
    const CsrMatrix *lhs_;
    lgx_direct *h_ = nullptr;
  };
  Instance instantiate(const CsrMatrix &lhs, const Environment &env) const {
    return Instance(lhs, env);
  }
};
using CholeskySolver = DenseDirectSolver<LGX_DIRECT_CHOLESKY>;
using LuSolver = DenseDirectSolver<LGX_DIRECT_LU>;
static_assert(DirectSolver<CholeskySolver> && DirectSolver<LuSolver>);

// ---- AMG (multigrid/*) -------------------------------------------------------------
enum struct CycleKind : uint8_t { REGULAR, DECREASING };
struct DefaultCycle {
  CycleKind kind = CycleKind::REGULAR;
  std::size_t iterations = 1;
};

struct HierarchyWrightParams {
  std::size_t max_level_num = 16;
  std::size_t min_coarsen_size = 2000;
  double min_coarsen_factor = 1.2;
};

struct AggregationParams {
  int32_t min_aggregate_size = 6;
  int32_t max_aggregate_size = 9;
  int64_t partition_size = 4096;
  double partition_growth = 4.0;
  int64_t min_partitions = 8;
  // RefinedAggregator::Params::base_agg_map_path (aggregation/independent.hpp:
  // 243-272): every level's aggregate map is written to <path><level>.aggs
  std::optional<std::string> base_agg_map_path{};
};

// ---- aggregate-map files (aggregation/independent.hpp:35-44, 237-298) ----------
// Both halves of lineal's BaseMultithreadAggregateMap (aggregate-map/
// multithread.hpp:299-303, 346-349).  lineal serialises them with its
// thesauros containers; the byte layout here is this library's own (the
// Python lineal_gb300.io module reads and writes the same files): 8 magic
// bytes "LGXAGGS1", u64 fine size n, u64 coarse size nc, u32 aggregate per
// fine vertex (0xFFFFFFFE: isolated), u64 list offsets[nc + 1], u32 fine
// vertex per list entry; little-endian.
struct AggregateMap {
  std::vector<uint32_t> agg;
  std::vector<int64_t> list_ptr{0};
  std::vector<int32_t> list;
  [[nodiscard]] lgx_agg_map view() const {
    return {(int64_t)agg.size(), (int64_t)list_ptr.size() - 1, agg.data(), list_ptr.data(),
            list.data()};
  }
};

inline std::string aggs_path(const std::string &base, std::size_t level) {
  return base + std::to_string(level) + ".aggs";
}

namespace detail {
inline constexpr char kAggsMagic[8] = {'L', 'G', 'X', 'A', 'G', 'G', 'S', '1'};
static_assert(std::endian::native == std::endian::little, "aggregate-map files are little-endian");

template <typename T>
void write_raw(std::FILE *f, const T *p, std::size_t n, const std::string &path) {
  if (n && std::fwrite(p, sizeof(T), n, f) != n)
    throw Error(LGX_ERR_INVALID, "lineal_gb300: cannot write " + path);
}
template <typename T>
void read_raw(std::FILE *f, T *p, std::size_t n, const std::string &path) {
  if (n && std::fread(p, sizeof(T), n, f) != n)
    throw Error(LGX_ERR_INVALID, "lineal_gb300: " + path + " is truncated");
}
struct File {
  std::FILE *f;
  ~File() {
    if (f) std::fclose(f);
  }
};
}  // namespace detail

// the checks lgx_agg_map_check applies (host only)
inline void check_aggregate_map(const AggregateMap &m) {
  if (m.list_ptr.empty() || (std::size_t)m.list_ptr.back() > m.list.size())
    throw Error(LGX_ERR_INVALID, "lineal_gb300: aggregate map offsets exceed its list");
  const lgx_agg_map v = m.view();
  check(lgx_agg_map_check(&v, v.n));
}

inline void write_aggs(const std::string &path, const AggregateMap &m) {
  check_aggregate_map(m);
  detail::File file{std::fopen(path.c_str(), "wb")};
  if (!file.f) throw Error(LGX_ERR_INVALID, "lineal_gb300: cannot open " + path);
  const uint64_t sizes[2] = {(uint64_t)m.agg.size(), (uint64_t)m.list_ptr.size() - 1};
  detail::write_raw(file.f, detail::kAggsMagic, 8, path);
  detail::write_raw(file.f, sizes, 2, path);
  detail::write_raw(file.f, m.agg.data(), m.agg.size(), path);
  detail::write_raw(file.f, m.list_ptr.data(), m.list_ptr.size(), path);
  const std::vector<uint32_t> list(m.list.begin(), m.list.begin() + m.list_ptr.back());
  detail::write_raw(file.f, list.data(), list.size(), path);
}

inline AggregateMap read_aggs(const std::string &path) {
  detail::File file{std::fopen(path.c_str(), "rb")};
  if (!file.f) throw Error(LGX_ERR_INVALID, "lineal_gb300: cannot open " + path);
  char magic[8];
  uint64_t sizes[2];
  detail::read_raw(file.f, magic, 8, path);
  if (!std::equal(magic, magic + 8, detail::kAggsMagic))
    throw Error(LGX_ERR_INVALID, "lineal_gb300: " + path + " is not an aggregate-map file");
  detail::read_raw(file.f, sizes, 2, path);
  if (sizes[0] > (uint64_t)INT32_MAX || sizes[1] > sizes[0])
    throw Error(LGX_ERR_INVALID, "lineal_gb300: " + path + " has impossible sizes");
  AggregateMap m;
  m.agg.resize(sizes[0]);
  m.list_ptr.resize(sizes[1] + 1);
  detail::read_raw(file.f, m.agg.data(), m.agg.size(), path);
  detail::read_raw(file.f, m.list_ptr.data(), m.list_ptr.size(), path);
  if (m.list_ptr.back() < 0 || (uint64_t)m.list_ptr.back() > sizes[0])
    throw Error(LGX_ERR_INVALID, "lineal_gb300: " + path + " has impossible list offsets");
  std::vector<uint32_t> list((std::size_t)m.list_ptr.back());
  detail::read_raw(file.f, list.data(), list.size(), path);
  if (std::fgetc(file.f) != EOF)
    throw Error(LGX_ERR_INVALID, "lineal_gb300: " + path + " is longer than its header says");
  m.list.assign(list.begin(), list.end());
  check_aggregate_map(m);
  return m;
}

// FileAggregator (aggregation/independent.hpp:279-298): the maps of levels
// 0, 1, ... up to the first missing file
inline std::vector<AggregateMap> read_aggregates(const std::string &base) {
  std::vector<AggregateMap> maps;
  for (;;) {
    const std::string path = aggs_path(base, maps.size());
    detail::File probe{std::fopen(path.c_str(), "rb")};
    if (!probe.f) break;
    maps.push_back(read_aggs(path));
  }
  if (maps.empty()) throw Error(LGX_ERR_INVALID, "lineal_gb300: no " + aggs_path(base, 0));
  return maps;
}

struct DuneDependencyCriterion {
  double strong_threshold = 1.0 / 3.0;
  double aggressive_strong_threshold = 1.0 / 3.0;
};

// MultiGridSolver{relax, DefaultCycle{REGULAR, 1}, wright} with lineal's
// default component choice: DuneDependencyCriterion + homogeneous greedy
// aggregation, SOR forward pre- and backward post-smoothing, direct coarsest
// solve (test/aux/default.hpp:155-188).
struct MultiGridSolver : SharedStationaryIterativeSolverBase {
  double relax = 1.0;
  DefaultCycle cycle{};
  HierarchyWrightParams hierarchy{};
  AggregationParams aggregation{};
  DuneDependencyCriterion criterion{};
  double smoother_relax = 1.0;
  bool float_cycle = false;
  bool bf16_values = false;  // with float_cycle: bfloat16 level values, diagonal row scales
  bool grid27 = true;        // 27-point grid finest level without column indices
  bool coarse_smallest_last = false;  // smallest-last colourings on levels >= 1
  // FileAggregator::Params::base_agg_map_path (aggregation/independent.hpp:
  // 279-298): when set, level k takes the aggregates of <path><k>.aggs
  std::optional<std::string> file_agg_map_path{};

  class Instance {
   public:
    Instance(const CsrMatrix &lhs, const MultiGridSolver &s, const Environment &env) {
      if (s.cycle.kind != CycleKind::REGULAR || s.cycle.iterations != 1)
        throw Error(LGX_ERR_UNSUPPORTED, "only the REGULAR cycle with one iteration (V-cycle)");
      lgx_amg_params p;
      lgx_amg_default_params(&p);
      p.max_level_num = (int64_t)s.hierarchy.max_level_num;
      p.min_coarsen_size = (int64_t)s.hierarchy.min_coarsen_size;
      p.min_coarsen_factor = s.hierarchy.min_coarsen_factor;
      p.min_aggregate_size = s.aggregation.min_aggregate_size;
      p.max_aggregate_size = s.aggregation.max_aggregate_size;
      p.partition_size = s.aggregation.partition_size;
      p.partition_growth = s.aggregation.partition_growth;
      p.min_partitions = s.aggregation.min_partitions;
      p.strong_threshold = s.criterion.strong_threshold;
      p.aggressive_threshold = s.criterion.aggressive_strong_threshold;
      p.relax = s.relax;
      p.smoother_relax = s.smoother_relax;
      p.cycle_f32 = s.float_cycle;
      p.cycle_bf16 = s.bf16_values;
      p.grid27 = s.grid27;
      p.coarse_smallest_last = s.coarse_smallest_last;
      if (s.file_agg_map_path) {
        const std::vector<AggregateMap> maps = read_aggregates(*s.file_agg_map_path);
        std::vector<lgx_agg_map> views;
        for (const auto &m : maps) views.push_back(m.view());
        check(lgx_amg_setup_given(lhs.handle(), &p, nullptr, views.data(), (int64_t)views.size(),
                                  env.stream(), &h_));
      } else {
        check(lgx_amg_setup(lhs.handle(), &p, nullptr, env.stream(), &h_));
      }
      if (s.aggregation.base_agg_map_path) {
        try {
          const std::size_t L = level_num();
          for (std::size_t l = 0; l + 1 < L; ++l)
            write_aggs(aggs_path(*s.aggregation.base_agg_map_path, l), aggregate_map(l, env));
        } catch (...) {
          lgx_amg_destroy(std::exchange(h_, nullptr));
          throw;
        }
      }
    }
    Instance(const Instance &) = delete;
    Instance(Instance &&o) noexcept : h_(std::exchange(o.h_, nullptr)) {}
    ~Instance() {
      if (h_) lgx_amg_destroy(h_);
    }
    static constexpr std::size_t in_situ_aux_size = 0;
    static constexpr std::size_t ex_situ_aux_size = 0;
    // apply(constant 0, out, rhs) -- the preconditioner application
    void apply(DenseVector<double> &out, const DenseVector<double> &rhs,
               const Environment &env) const {
      check(lgx_amg_vcycle(h_, rhs.data(), out.data(), env.stream()));
    }
    // lineal's call shape apply(constant_like(out, 0), out, rhs, aux, env)
    // (multigrid/solver.hpp:41-56); the cycle starts from zero only
    template <typename TAux>
    void apply(const ConstantExpr &in, DenseVector<double> &out, const DenseVector<double> &rhs,
               TAux && /*aux*/, const Environment &env) const {
      if (in.value != 0.0 || in.size != out.size())
        throw Error(LGX_ERR_UNSUPPORTED,
                    "lineal_gb300: MultiGridSolver applies from a zero initial guess");
      apply(out, rhs, env);
    }
    [[nodiscard]] lgx_amg *handle() const { return h_; }
    // level l's aggregates (lgx_amg_level_download + lgx_amg_level_lists)
    [[nodiscard]] AggregateMap aggregate_map(std::size_t l, const Environment &env) const {
      int64_t L = 0;
      std::vector<int64_t> rows(64), nnz(64);
      check(lgx_amg_info(h_, &L, rows.data(), nnz.data(), (int64_t)rows.size()));
      if ((int64_t)l + 1 >= L) throw Error(LGX_ERR_INVALID, "lineal_gb300: level has no map");
      AggregateMap m;
      m.agg.resize((std::size_t)rows[l]);
      m.list_ptr.resize((std::size_t)rows[l + 1] + 1);
      check(lgx_amg_level_download(h_, (int64_t)l, nullptr, nullptr, nullptr, m.agg.data(),
                                   env.stream()));
      int64_t len = 0;
      check(lgx_amg_level_lists(h_, (int64_t)l, m.list_ptr.data(), nullptr, &len, env.stream()));
      m.list.resize((std::size_t)len);
      check(lgx_amg_level_lists(h_, (int64_t)l, nullptr, m.list.data(), nullptr, env.stream()));
      return m;
    }
    [[nodiscard]] std::size_t level_num() const {
      int64_t l = 0;
      check(lgx_amg_info(h_, &l, nullptr, nullptr, 0));
      return (std::size_t)l;
    }
    // times the row-kernel shapes of every level and keeps the fastest
    // (lgx_amg_autotune); returns the per-level report
    std::vector<lgx_tune_entry> autotune(const Environment &env, int reps = 3) {
      std::vector<lgx_tune_entry> out(2 * level_num() + 1);
      int n = 0;
      check(lgx_amg_autotune(h_, reps, out.data(), (int)out.size(), &n, env.stream()));
      out.resize(std::min<std::size_t>((std::size_t)n, out.size()));
      return out;
    }

   private:
    lgx_amg *h_ = nullptr;
  };

  Instance instantiate(const CsrMatrix &lhs, const Environment &env) const {
    return Instance(lhs, *this, env);
  }
};

// ---- non-stationary solvers ----------------------------------------------------------
struct NoPrecon {};

// ConjugateGradientsSolver / BiCgStabSolver (conjugate-gradients/solver.hpp:24-225,
// bicgstab/solver.hpp:25-263).  TPrecon is void, JacobiSolver, MultiGridSolver.
template <lgx_krylov_kind tKind, typename TPrecon>
struct KrylovSolver : SharedNonStationaryIterativeSolverBase {
  std::size_t rere_period = 8;  // rere_controller: iter > 0 && iter % 8 == 0
  std::optional<TPrecon> precon;
  bool flexible = false;        // CG: flexible beta (float V-cycle preconditioners)

  KrylovSolver() = default;
  explicit KrylovSolver(TPrecon p, std::size_t rere = 8) : rere_period(rere), precon(std::move(p)) {}

  template <AnyMatrix TLhs>
  struct Instance {
    const TLhs &lhs;
    const KrylovSolver &solver;
    std::optional<MultiGridSolver::Instance> amg;

    struct SystemInstance {
      SystemInstance(const Instance &inst, DenseVector<double> &sol,
                     const DenseVector<double> &rhs, const Environment &env)
          : sol_(sol) {
        lgx_solve_params p;
        lgx_solve_default_params(&p);
        p.rere_period = (int64_t)inst.solver.rere_period;
        p.flexible = inst.solver.flexible ? 1 : 0;
        if constexpr (std::is_same_v<TPrecon, JacobiSolver>) {
          p.precon = LGX_PRECON_JACOBI;
          p.relax = inst.solver.precon->relax;
        } else if constexpr (std::is_same_v<TPrecon, MultiGridSolver>) {
          p.precon = LGX_PRECON_AMG;
          p.amg = inst.amg->handle();
        }
        check(lgx_krylov_create(tKind, inst.lhs.handle(), rhs.data(), sol.data(), &p,
                                env.stream(), &h_));
      }
      SystemInstance(const SystemInstance &) = delete;
      ~SystemInstance() {
        if (h_) lgx_krylov_destroy(h_);
      }
      void iterate(const Environment & /*env*/) { check(lgx_krylov_iterate(h_)); }
      [[nodiscard]] double residual_norm() const { return state().res; }
      [[nodiscard]] double rho() const { return state().rho; }
      [[nodiscard]] const DenseVector<double> &solution() {
        check(lgx_krylov_solution(h_, sol_.data()));
        return sol_;
      }

     private:
      struct St {
        int64_t it;
        double res, rho;
      };
      [[nodiscard]] St state() const {
        St s{};
        check(lgx_krylov_state(h_, &s.it, &s.res, &s.rho));
        return s;
      }
      lgx_krylov *h_ = nullptr;
      DenseVector<double> &sol_;
    };

    SystemInstance instantiate(DenseVector<double> &sol, const DenseVector<double> &rhs,
                               const Environment &env) const {
      return SystemInstance(*this, sol, rhs, env);
    }
  };

  template <AnyMatrix TLhs>
  Instance<TLhs> instantiate(const TLhs &lhs, const Environment &env) const {
    Instance<TLhs> inst{lhs, *this, std::nullopt};
    if constexpr (std::is_same_v<TPrecon, MultiGridSolver>) inst.amg.emplace(lhs, *precon, env);
    return inst;
  }
};

template <typename TPrecon = void>
using ConjugateGradientsSolver =
  KrylovSolver<LGX_KRYLOV_CG, std::conditional_t<std::is_void_v<TPrecon>, NoPrecon, TPrecon>>;
template <typename TPrecon = void>
using BiCgStabSolver =
  KrylovSolver<LGX_KRYLOV_BICGSTAB, std::conditional_t<std::is_void_v<TPrecon>, NoPrecon, TPrecon>>;

// run_iterative_solver (linear-solver/runner.hpp:17-84): the caller's iter_op
// decides when to stop and returns the value to report.
template <typename TSolver, AnyMatrix TLhs, typename TIterOp>
auto run_iterative_solver(const TSolver &solver, const TLhs &lhs, DenseVector<double> &sol,
                          const DenseVector<double> &rhs, const Environment &env,
                          TIterOp iter_op) {
  auto instance = solver.instantiate(lhs, env);
  auto system = instance.instantiate(sol, rhs, env);
  if (auto r = iter_op(std::size_t{0}, system, env); r.has_value()) {
    (void)system.solution();
    return *r;
  }
  for (std::size_t i = 1;; ++i) {
    system.iterate(env);
    if (auto r = iter_op(i, system, env); r.has_value()) {
      (void)system.solution();
      return *r;
    }
  }
}

}  // namespace lineal::gb300
