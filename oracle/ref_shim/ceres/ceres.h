// Minimal stand-in for the parts of Ceres Solver that painty's PaintMixer.cxx names, written for
// this repository so that file compiles unmodified in the oracle build (Ceres is not installed
// here). It declares the types and calls the mixer's fitting routines use; Solve() leaves the
// parameters where they are. Only PaintMixer::mixSinglePaint, which calls no Ceres code, is
// exercised through it.
#pragma once
#include <cmath>
#include <memory>
#include <vector>

namespace ceres {

template <typename T>
T abs(const T& x) { return std::abs(x); }
template <typename T>
T exp(const T& x) { return std::exp(x); }
template <typename T>
T cosh(const T& x) { return std::cosh(x); }
template <typename T>
T sinh(const T& x) { return std::sinh(x); }
template <typename T>
T sqrt(const T& x) { return std::sqrt(x); }
template <typename T, typename U>
T pow(const T& x, const U& y) { return std::pow(x, y); }

enum Ownership { DO_NOT_TAKE_OWNERSHIP = 0, TAKE_OWNERSHIP = 1 };

class CostFunction {
 public:
  virtual ~CostFunction() = default;
  void SetNumResiduals(int n) { num_residuals_ = n; }
  void AddParameterBlock(int size) { blocks_.push_back(size); }

 private:
  int num_residuals_ = 0;
  std::vector<int> blocks_;
};

template <typename Functor, int Stride = 4>
class DynamicAutoDiffCostFunction : public CostFunction {
 public:
  explicit DynamicAutoDiffCostFunction(Functor* f) : functor_(f) {}

 private:
  std::unique_ptr<Functor> functor_;
};

class LossFunction {
 public:
  virtual ~LossFunction() = default;
};

class ScaledLoss : public LossFunction {
 public:
  ScaledLoss(const LossFunction* rho, double a, Ownership ownership)
      : rho_(rho), a_(a), ownership_(ownership) {}

 private:
  const LossFunction* rho_;
  double a_;
  Ownership ownership_;
};

// Holds nothing: the stand-in only has to compile the fitting routines, which the oracle
// build never runs.
class Problem {
 public:
  template <typename... Blocks>
  void AddResidualBlock(CostFunction*, LossFunction*, Blocks*...) {}
  void SetParameterLowerBound(double*, int, double) {}
  void SetParameterUpperBound(double*, int, double) {}
};

struct Solver {
  struct Options {
    bool minimizer_progress_to_stdout = false;
    int num_threads = 1;
    int num_linear_solver_threads = 1;
    int max_num_iterations = 50;
    double function_tolerance = 1e-6;
  };
  struct Summary {};
};

inline void Solve(const Solver::Options&, Problem*, Solver::Summary*) {}

}  // namespace ceres
