// GPU recursive-skeletonization factorization: host-side orchestration.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <string>
#include <array>
#include <functional>
#include <vector>

#include "ki_tree.h"

namespace ki {

struct Params {
  int dim = 2;                // domain dimension: 2 or 3
  int sol_dim = 1;            // 1: Laplace, 2: Stokes (2D), 3: Stokes (3D)
  int pde = 0;                // 2D scalar kernel (Points::pde): 0, kPdeNeumann, kPdeGauss
  int max_leaf_dofs = 64;     // MAX_LEAF_DOFS
  int num_proxy_points = 128; // NUM_PROXY_POINTS (2D); 3D: theta x phi grid, 2 q^2 points
  double radius_ratio = 2.0;  // RADIUS_RATIO: proxy radius = ratio*sqrt(dim)*side/2
  int min_dofs_to_compress = 64;
  double id_tol = 1e-10;
  // learned rank predictor (device model blob, ki_mlp.h) or null: with a model
  // the ID of every box whose triangle fits in shared memory is a sketched ID
  // of l = min(n, ceil((1 + sketch_margin) k^) + sketch_oversample) rows
  const float* rank_model = nullptr;
  float sketch_margin = 0.25f;
  int sketch_oversample = 8;
};

// Device status word written by kernels that can fail (non-finite data,
// singular pivot); read back by the host after each stage.
enum DeviceError : int { kDevOk = 0, kDevNonFinite = 1, kDevSingular = 2, kDevTimeout = 3 };

// Per-level description of the compressed boxes, kept for the solve sweeps.
struct LevelFactor {
  int n_comp = 0;          // compressed boxes in this level
  void* d_tasks = nullptr; // device array of per-box sweep descriptors
  int max_n = 0;           // largest active set among them
  int max_mat = 0;         // largest factor matrix among them: max(r^2, k r) entries
  int max_all = 0;         // largest 2 k r + r^2 (every factor matrix of a box)
  double sum_kr = 0, sum_r2 = 0, sum_n = 0, sum_r = 0;   // over the compressed boxes (sweep work)
};

// Per box of the tree, the factors a later re-factorization of a perturbed
// boundary copies instead of recomputing (SkelFactorization::skeletonize
// skips boxes still `compressed` after QuadTree::perturb,
// kern_interp/skel_factorization/skel_factorization.cpp:199-208).
template <typename T>
struct BoxFactor {
  int n = 0;                 // active DOFs at the box's level
  int k = 0;                 // skeleton size (compressed boxes)
  bool compressed = false;
  int64_t pact = 0;          // pool offset of the permuted active list (skeleton first)
  const T* tile = nullptr;   // compressed: Schur-updated skeleton block K~ss (k x k)
  const T* Tm = nullptr;     // interpolation matrix (k x r)
  const T* L = nullptr;      // k x r
  const T* U = nullptr;      // r x k
  const T* X = nullptr;      // LU of the redundant block (r x r)
  const int* piv = nullptr;  // its pivots (r)
  const T* Xi = nullptr;     // explicit inverse of the redundant block (FP32) or null
};

// Device-time record of one launch group (CUDA events on the factor's stream).
struct StageRec {
  std::string stage;
  cudaEvent_t a = nullptr, b = nullptr;
  double flops = 0;     // algorithmic flops of the launch
  double bytes = 0;     // algorithmic bytes of the launch
};

struct StageSum {
  std::string stage;
  int launches = 0;
  double ms = 0, flops = 0, bytes = 0;
};

// Per-level shape statistics of the compressed boxes.
struct LevelStat {
  int level = 0, boxes = 0, id_boxes = 0, compressed = 0;
  int max_n = 0, max_m = 0, max_k = 0;
  double sum_n = 0, sum_m = 0, sum_k = 0;
  // narrow/smem, narrow/global, wide/smem, wide/global, narrow with a
  // tensor-core sketch
  int mode_count[5] = {0, 0, 0, 0, 0};
};

template <typename T>
struct Factorization {
  Params prm;
  Tree tree;
  cudaStream_t stream = nullptr;
  // auxiliary streams: independent launch groups of a level run concurrently
  static constexpr int kAux = 4;
  cudaStream_t aux[kAux] = {};
  cudaEvent_t fork_ev = nullptr, join_ev[kAux] = {};
  void fork();                        // aux streams wait for `stream`
  void join(int used);                // `stream` waits for aux[0..used)
  // every launch group on `stream` (the autotuner's timing runs: each
  // group's events then time it alone)
  bool serial = false;
  int N = 0;           // DOFs
  int n_points = 0;
  // point data (device, SoA, precision T)
  T *d_x = nullptr, *d_y = nullptr, *d_nx = nullptr, *d_ny = nullptr, *d_w = nullptr,
    *d_kappa = nullptr, *d_z = nullptr, *d_nz = nullptr;
  // FP32 form: low parts of the coordinates (nullptr in FP64)
  T *d_xl = nullptr, *d_yl = nullptr, *d_zl = nullptr;
  // 3D diagonal entries (Kernel::compute_diag_entries_3dlaplace/_3dstokes):
  // FP64 (kept for the FP64 operator apply) and in the factor precision
  double* d_diag64 = nullptr;
  T* d_diag = nullptr;
  int diag_per_point = 0;   // 1 (Laplace), 9 (Stokes), 0 in 2D
  std::vector<LevelFactor> levels;   // index = tree level
  // every level's sweep descriptors in one device array, ascending active
  // size, for the diagonal solves of all levels in one pass; bins of boxes
  // launched together
  void* d_all_tasks = nullptr;
  std::vector<std::array<int, 4>> diag_bins;   // {first, count, largest n, largest r^2}
  // root
  int n_root = 0;
  int* d_root_idx = nullptr;  // allskel DOF list
  T* d_root_lu = nullptr;     // LU of the root block (or the bordered S)
  int* d_root_piv = nullptr;
  int n_border = 0;           // border columns (holes x c)
  int n_root_sys = 0;         // n_root + n_border
  // bordered data (multiply connected)
  T* d_Umod = nullptr;        // N x nb, DOF-major: swept U
  T* d_PsiTmod = nullptr;     // N x nb, DOF-major: swept Psi^T
  T* d_DinvU = nullptr;       // N x nb, DOF-major: D^-1 U~ on the redundant rows
  unsigned char* d_is_skel = nullptr;  // N flags
  int* d_err = nullptr;       // device status word
  // statistics
  int n_compressed = 0;
  long n_redundant = 0;
  int n_sketched = 0;                // boxes compressed from a sketch
  int n_fallback = 0;                // sketches that did not reveal the rank
  std::vector<float> box_log;        // per ID box: 12 features, n, k, level
  std::vector<int> rank_hist;
  bool profile_solve = false;        // record stage events in solves
  std::vector<StageRec> prof_open;   // launches recorded since the last collect
  std::vector<size_t> prof_stack;    // open stages (nested begin/end pairs)
  std::vector<StageSum> factor_prof; // per stage, factorization
  std::vector<LevelStat> level_stats;
  std::vector<StageSum> solve_prof;  // per stage, last solve
  void stage_begin(const char* name, double flops, double bytes, cudaStream_t on = nullptr);
  void stage_end(cudaStream_t on = nullptr);
  std::vector<StageSum> collect();   // synchronizes the stream
  double factor_seconds = 0;
  double tree_seconds = 0;   // tree build (codes on the GPU, boxes on the host)
  bool tree_gpu = false;      // the tree was built on the GPU (else by the host partition)
  double tree_codes_seconds = 0;   // from the start of the factorization to the GPU-built tree on the host
  size_t device_bytes = 0;
  std::vector<void*> owned;   // device allocations to free
  // re-factorization: every box's factors (index = box of `tree`), the
  // integer pool their lists live in, and how many boxes this factorization
  // copied from the one it updated
  std::vector<BoxFactor<T>> box_factors;
  const int* d_ipool = nullptr;
  int n_reused = 0;

  ~Factorization();
  void* alloc(size_t bytes);
};

// Border columns per hole of the bordered system (initialize_U_mat,
// kern_interp/linear_solve.cpp:19-107): Laplace 1, 2D Stokes 3 (Stokeslet x2
// + rotlet), 3D Stokes 6 (Stokeslet x3 + rotlet x3).
__host__ __device__ inline int border_cols_per_hole(int dim, int sol_dim) {
  return sol_dim == 1 ? 1 : (dim == 2 ? 3 : 6);
}

struct HoleDesc {
  int n_holes = 0;
  std::vector<double> centers;   // dim per hole
  std::vector<int> start, count; // node ranges
};

// Build the tree and skeletonize on `stream`.  Throws std::runtime_error on
// failure (message says which stage).
template <typename T>
// after_tree (optional): called once the tree is built (the host work the
// caller defers until the tree no longer competes for the CPU cores).
// d_inputs (optional): the same four arrays already on the device, laid out
// points (dim n) | normals (dim n) | weights (n) | curvatures (n), kept alive
// by the caller for the factorization's lifetime; otherwise they are copied.
// prev (optional): a factorization of the same problem before a boundary
// perturbation (QuadTree::perturb, kern_interp/quadtree/quadtree.cpp:581-890).
// A box whose active DOFs, their data (the precision-T point arrays the
// kernels read) and its near field are unchanged -- it has a box of prev's
// tree at the same level and centre, the same leaf DOF list or the same
// reused children, and neighbours that are unchanged in the same sense --
// gets prev's factors copied instead of an ID and a Schur elimination.  Used
// only when prev has the same number of points and the same parameters;
// prev must stay alive until this returns.
std::unique_ptr<Factorization<T>> factorize(const Params& prm, int n_points, const double* points,
                                            const double* normals, const double* weights,
                                            const double* curvatures, const HoleDesc& holes,
                                            cudaStream_t stream,
                                            const double* d_inputs = nullptr,
                                            const std::function<void()>& after_tree = nullptr,
                                            const Factorization<T>* prev = nullptr);

// A bump allocator over caller-provided device memory.
struct ScratchArena {
  char* base = nullptr;
  size_t size = 0, used = 0;
  void* take(size_t bytes) {
    size_t off = (used + 255) & ~size_t(255);
    if (off + bytes > size) return nullptr;
    used = off + bytes;
    return base + off;
  }
};

// Runs the tensor-core sketch machinery (tcgen05 TF32 MMAs, TMEM
// accumulators) on fixed data on the current device and returns its largest
// difference from the same product in FP64, relative to the largest entry.
double tensor_core_selfcheck();

// Device bytes solve_device_arena takes from its arena for ncols columns
// (including 256-byte alignment of every piece).
template <typename T>
size_t solve_arena_bytes(const Factorization<T>& F, int ncols);

// solve_device with every temporary taken from `arena` (no allocation, no
// profiling events); `s` is the stream of the whole solve.
template <typename T>
void solve_device_arena(Factorization<T>& F, T* d_x, int ncols, T* d_alpha, ScratchArena& arena,
                        cudaStream_t s);

// Solve with the factorization: x (device, DOF-major N x ncols, ld = ncols)
// is overwritten with the solution; alpha (device, n_border x ncols,
// row-major) receives the border unknowns of a multiply connected problem.
// g (optional, row-major n_border x ncols): right-hand side of the border
// rows, Psi mu - alpha = g (zero in the reference's problem; refinement
// corrections carry one).
template <typename T>
void solve_device(Factorization<T>& F, T* d_x, int ncols, T* d_alpha, const T* d_g = nullptr);

}  // namespace ki
