// Declarations of the two Ceres names the reference's
// utils/camera/SnavelyReprojectionError.h refers to, so the reference's
// functor compiles without Ceres.  TEST INFRASTRUCTURE (oracle/_ref only):
// nothing here differentiates or solves.
#pragma once
namespace ceres {
class CostFunction {
 public:
  virtual ~CostFunction() {}
};
template <typename Functor, int kNumResiduals, int... Ns>
class AutoDiffCostFunction : public CostFunction {
 public:
  explicit AutoDiffCostFunction(Functor *f) : functor(f) {}
  ~AutoDiffCostFunction() override { delete functor; }
  Functor *functor;
};
}  // namespace ceres
