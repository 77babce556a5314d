// Internal declarations shared by the CUDA translation units of the kernel
// layer (not part of the public C-ABI).
#pragma once
#include <cuda_runtime.h>
#include <functional>
#include "starpu_gb300_kernels.h"
#include "starpu_gb300_solver.h"

namespace gb300 {

// largest diagonal tile the cooperative factor-and-invert kernel handles
constexpr int GB300_DIAG_TILE_MAX = 1024;

// residual partials P_z = -(A X) on the tensor cores (capi_tc.cu)
size_t residual_tc_a_bytes(int n);
int residual_tc_slice_a(cudaStream_t s, int n, const double *A, long lda, const unsigned long long *amax_bits,
                        void *slices, float *rowsum);
size_t residual_tc_xs_bytes(int n, int nrhs);
int residual_tc_kchunk(int n, int nrhs, int max_chunks);
int residual_tc(cudaStream_t s, int n, int nrhs, const void *a_slices, const double *X, long ldx, const int *sx,
                const unsigned long long *anorm_bits, int kchunk, void *xs, double *partials, int *d_err);


// Columns of the matrix arriving while the tensor-core factorisation runs
// (the host-buffer solve gathers A over the host link superblock by
// superblock): superblock s holds columns [start[s], start[s + 1]) of W (rows
// >= start[s]) once ready[s] has completed; diag is the diagonal of A (n
// floats), complete before the factorisation starts; panel_store holds every
// step's split panel (tc_arrival_store_bytes), which the updates of columns
// that arrive late replay in step order.  The result is bit-identical to
// the factorisation of the whole matrix.
struct TcArrival {
    int nsb = 0;
    const int *start = nullptr;
    const cudaEvent_t *ready = nullptr;
    const float *diag = nullptr;
    void *panel_store = nullptr;
    int lookahead_blocks = 2;  // superblocks are taken in this many column blocks ahead of need
};
size_t tc_arrival_store_bytes(int n, int nb);
int potrf_tc(cudaStream_t s, int n, float *A, long lda, int nb, int nterms, void *panel, int *d_info, int *d_err,
             float *linv_band, const std::function<void(cudaStream_t)> &side, int side_rows,
             const std::function<void(cudaStream_t, int, int)> &on_panel, cudaEvent_t ready,
             const TcArrival *arr = nullptr);

// the two phases of starpu_gb300_dsposv (capi_solver.cu)
// prepared: W (FP32 lower A) and max |A_ij| are already in the workspace
int dsposv_factor(cudaStream_t s, int n, int nrhs, const double *A, int lda, int nb, int nterms, void *work,
                  starpu_gb300_ir_info *out, bool prepared = false, const TcArrival *arr = nullptr);
// the workspace regions the host path's fused gather writes: W (n x n FP32)
// and the word that receives max |A_ij| (zeroed with its three neighbours)
void dsposv_prepared_targets(int n, int nrhs, int nb, void *work, float **W, unsigned long long **amax_block);
// stalled (optional): set when the refinement stopped without converging
int dsposv_refine(cudaStream_t s, int n, int nrhs, const double *A, int lda, const double *B, int ldb, double *X,
                  int ldx, int nb, double tol, int max_iter, void *work, starpu_gb300_ir_info *out,
                  bool *stalled = nullptr);
// LAPACK dsposv's fallback: FP64 factorisation and solve of A on the GPU
int dsposv_fp64(cudaStream_t s, int n, int nrhs, const double *A, int lda, const double *B, int ldb, double *X,
                int ldx, int nb, double tol, void *work, starpu_gb300_ir_info *out);
// factor + refinement, then the FP64 fallback when either fails
int dsposv_ladder(cudaStream_t s, int n, int nrhs, const double *A, int lda, const double *B, int ldb, double *X,
                  int ldx, int nb, int nterms, double tol, int max_iter, void *work, starpu_gb300_ir_info *out,
                  bool prepared, const TcArrival *arr = nullptr);

// The mixed solve's schedule for one tile size, from starpu_gb300_dense_autotune,
// stored in the tuning table beside the perfmodels (capi_batched.cu).
struct DenseTuning {
    int nb = 0;
    int lookahead_sms = -1;     // -1: chosen per step by the model below
    double t_diag_us = 0;       // diagonal-tile factor + inverse on a quarter of the SMs
    double update_tflops = 0;   // the split-precision trailing update on the whole GPU
    double panel_rate = 0;      // the panel solve's tensor rate per SM, relative to the update's
    int n = 0;                  // order the schedule was timed at
    double step_ms = 0;         // its factorisation time
};
bool dense_tuning(int nb, DenseTuning *out);
int dense_tuning_store(const DenseTuning &d);

// Width of the register-blocked small triangular kernels and of the
// unblocked diagonal POTRF leaf: 64 columns in FP32, 32 in FP64 (a 64-wide
// FP64 row does not fit the register file without spilling).
template <typename T> struct small_w { static constexpr int value = 64; };
template <> struct small_w<double> { static constexpr int value = 32; };

template <typename T>
void gemm(cudaStream_t s, bool ta, bool tb, bool lower, int m, int n, int k, T alpha, const T *A, long lda,
          const T *B, long ldb, T beta, T *C, long ldc);
template <typename T> void trsm_rltn(cudaStream_t s, int m, int nc, const T *L, long ldl, T *B, long ldb);
template <typename T> void potrf_tiled(cudaStream_t s, int n, T *A, long lda, int nb, int *info, int info_base);
// Linv = inverse of the lower triangle of L (n x n, ld ldi, upper part zeroed); scratch >= n*n/4 elements
template <typename T> void trtri_lower(cudaStream_t s, int n, const T *L, long ldl, T *Linv, long ldi, T *scratch);
template <typename T> void potrs_blocked(cudaStream_t s, int n, int nrhs, const T *L, long ldl, T *B, long ldb);
// single-launch sweeps: workspace = inverted 64x64 diagonal blocks + flags
template <typename T> size_t potrs_sweep_workspace(int n);
template <typename T> void potrs_sweep_prepare(cudaStream_t s, int n, const T *L, long ldl, void *ws);
template <typename T>
void potrs_sweep(cudaStream_t s, int n, int nrhs, const T *L, long ldl, void *ws, T *B, long ldb, int *err);

} // namespace gb300

// Records the CUDA error (if any) of the most recent launch in this thread and
// maps it to a GB300_* return code.
extern "C" int gb300_last_launch_status(void);
extern "C" int gb300_record_cuda_error(cudaError_t e);
// Sets the message returned by starpu_gb300_last_error() for a non-CUDA error.
extern "C" void gb300_set_error(const char *msg);

// Every kernel launch site of the library calls this (it feeds
// starpu_gb300_launch_count()).
extern "C" void gb300_count_launch(void);

// Raise fn's dynamic shared memory limit to `bytes` on the current device,
// once per (function, device); returns a GB300_* code.
extern "C" int gb300_func_dyn_smem(const void *fn, int bytes);
// Multiprocessor count of the current device (cached per device).
extern "C" int gb300_device_sms(void);
// Limit of one bounded wait on a flag or counter written by another CTA of
// the same launch (starpu_gb300_set_wait_budget_ns; default 2 s).
extern "C" unsigned long long gb300_wait_budget_ns(void);

// Per-kernel-class timing (the profiling mode of starpu_gb300_profiling_*):
// prof_begin/prof_end bracket one launch with CUDA events on its stream when
// profiling is enabled; both are no-ops otherwise.
enum gb300_prof_kind { GB300_PROF_TC_UPDATE = 0, GB300_PROF_PANEL = 1, GB300_PROF_RESIDUAL = 2, GB300_PROF_SOLVE = 3,
                       GB300_PROF_BATCHED = 4, GB300_PROF_TRANSFER = 5, GB300_PROF_KINDS = 6 };
extern "C" int gb300_prof_begin(cudaStream_t s, int kind);
extern "C" void gb300_prof_end(cudaStream_t s, int slot, double algorithmic_flops, double algorithmic_bytes);
// the fraction of the SMs a profiled launch was limited to (default 1)
extern "C" void gb300_prof_set_share(int slot, double sm_share);
