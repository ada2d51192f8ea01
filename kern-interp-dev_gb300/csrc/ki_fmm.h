// Fast FP64 apply of the 2D Laplace double-layer Nystrom operator by a
// uniform-depth fast multipole method, for the residuals of iterative
// refinement.
//
// The operator is the reference's (Kernel::one_d_kern, kern_interp/kernel/
// kernel.cpp:33-43): K(t, s) = -w_s/(2 pi) (r . n_s)/|r|^2, r = t - s, and the
// curvature limit 1/2 + kappa_t w_t/(4 pi) on the diagonal.  With complex
// coordinates, (r . n_s)/|r|^2 = Re(n_s / (t - s)), so
//   (K mu)(t) = diag_t mu_t + Re sum_{s != t} q_s / (t - s),
//   q_s = -(w_s / 2 pi) n_s mu_s,
// a Cauchy sum: multipole (Laurent) expansions about box centres, local
// (Taylor) expansions, and the classical translations.  Expansions are
// scaled by the box side so every translation matrix has entries below one.
#pragma once

#include <cuda_runtime.h>

#include <memory>

namespace ki {

struct Fmm2d;
struct Fmm2dPlan;

struct Fmm2dDeleter {
  void operator()(Fmm2d* f) const;
};
struct Fmm2dPlanDeleter {
  void operator()(Fmm2dPlan* f) const;
};

// Host part of the build: tree, lists and translation matrices for n points
// (interleaved FP64 host arrays) with p expansion terms.  Pure host work,
// safe on a worker thread.  Throws std::invalid_argument.
std::unique_ptr<Fmm2dPlan, Fmm2dPlanDeleter> fmm2d_plan(const double* points,
                                                        const double* normals,
                                                        const double* weights,
                                                        const double* curvatures, int n, int p);

// Device part: upload a plan.  Throws std::runtime_error.
std::unique_ptr<Fmm2d, Fmm2dDeleter> fmm2d_upload(const Fmm2dPlan& plan, cudaStream_t s);

// Both steps.
std::unique_ptr<Fmm2d, Fmm2dDeleter> fmm2d_build(const double* points, const double* normals,
                                                 const double* weights, const double* curvatures,
                                                 int n, int p, cudaStream_t s);

// Optional recorder of the apply's launch groups (CUDA events on the apply's
// stream), with their algorithmic flops.
struct StageRecorder {
  virtual void begin(const char* name, double flops) = 0;
  virtual void end() = 0;
  virtual ~StageRecorder() = default;
};

// Arithmetic of the expansions and the near-field sums.  kF32: charges,
// expansions, translations and near-field sums in FP32 (point differences
// from hi/lo FP32 pairs, the diagonal term and the output in FP64), a
// relative error near 1e-6 -- for applies whose result only needs that
// accuracy (the residual updates of refinement, where the input is a small
// correction).
enum class FmmArith { kF64, kF32 };

// y (n x ncols, column-major, ldy) = K mu (n x ncols, ldmu), device buffers,
// on stream s, with `order` <= the plan's expansion terms (0: all of them);
// the translation matrices of a lower order are leading blocks of the
// plan's.  Stages recorded: fmm_upward (charges, P2M, M2M), fmm_m2l, fmm_l2l,
// fmm_near (local expansions at the targets and the direct near field);
// with the prefix fmm32_ for kF32.
void fmm2d_apply(Fmm2d& f, const double* mu, int ldmu, int ncols, double* y, int ldy,
                 cudaStream_t s, int order = 0, StageRecorder* rec = nullptr,
                 FmmArith arith = FmmArith::kF64);

// Expansion terms the plan was built with.
int fmm2d_order(const Fmm2d& f);

// Tree statistics (for reports): leaf level, leaves, boxes, M2L pairs,
// near-field leaf pairs.
void fmm2d_stats(const Fmm2d& f, int* level, int* leaves, int* boxes, long* m2l_pairs,
                 long* near_pairs);

}  // namespace ki
