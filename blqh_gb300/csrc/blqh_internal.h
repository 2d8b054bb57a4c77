// Internal declarations shared by the CUDA translation units of libblqh_gpu.so.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/blqh_gpu.h"

#define BLQH_MAX_NPHI 16   // 2*nphi bits per spinless state; the index tables are sized 2^nphi
#define BLQH_MAX_LAMBDA 4096

// ---------------------------------------------------------------------------
// error handling: every API call returns a status; the message is kept per
// context and per thread.
struct BlqhError {
  int code;
  std::string msg;
};
void set_error(blqh_ctx* ctx, int code, const std::string& msg);
#define BLQH_TRY_CUDA(ctx, expr)                                                        \
  do {                                                                                  \
    cudaError_t e_ = (expr);                                                            \
    if (e_ != cudaSuccess) {                                                            \
      set_error((ctx), BLQH_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(e_)); \
      throw BlqhError{BLQH_ERR_CUDA, cudaGetErrorString(e_)};                           \
    }                                                                                   \
  } while (0)

// ---------------------------------------------------------------------------
// timers: device time per kernel class, measured with events on the context
// stream when enabled (0 SpMV, 1 reorthogonalization, 2 CSR build and Rayleigh
// regeneration, 3 basis, 4 everything else).
enum { TM_SPMV = 0, TM_REORTH = 1, TM_BUILD = 2, TM_BASIS = 3, TM_MISC = 4, TM_N = 5 };

struct blqh_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  bool timing = false;
  double ms[TM_N] = {0, 0, 0, 0, 0};
  int64_t launches[TM_N] = {0, 0, 0, 0, 0};
  cudaEvent_t marks[8] = {};
  std::vector<cudaEvent_t> ev_pool;
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> pending;
  // small pinned host buffer for scalar read-backs
  double* pinned = nullptr;
};

// Device allocation that throws BlqhError on failure. Blocks are cached per
// context after dev_free (see runtime.cu); dev_forget_ctx releases a context's.
void* dev_alloc(blqh_ctx* ctx, size_t bytes);
void dev_free(void* p);
void dev_forget_ctx(blqh_ctx* ctx);
template <class T>
T* dalloc(blqh_ctx* ctx, size_t n) {
  return static_cast<T*>(dev_alloc(ctx, n * sizeof(T) + 16));
}
// Scratch device buffers of one call, released (dev_free) when the holder goes out of scope.
struct DevBufs {
  std::vector<void*> ps;
  DevBufs() = default;
  DevBufs(const DevBufs&) = delete;
  DevBufs& operator=(const DevBufs&) = delete;
  ~DevBufs() {
    for (void* p : ps) dev_free(p);
  }
  template <class T>
  T* add(T* p) {
    ps.push_back(p);
    return p;
  }
};

// Kernel-class timing brackets (no-ops unless timing is enabled).
struct TimerScope {
  blqh_ctx* ctx;
  int cls;
  cudaEvent_t a = nullptr, b = nullptr;
  TimerScope(blqh_ctx* c, int k);
  ~TimerScope();
};
void count_launch(blqh_ctx* ctx, int cls, int n = 1);
void flush_timers(blqh_ctx* ctx);

// ---------------------------------------------------------------------------
// Sector index: a dense numbering of the states that pass the momentum filter,
// equal to the order in which the reference's depth-first enumeration inserts
// them (basis.cpp:199-259). Tables live in device memory; the struct is passed
// to kernels by value.
struct SectorIdx {
  int nphi, nel, nel_up, nel_dn, J, K;
  int all_density;  // nel_up < 0: free layer split
  uint32_t lmask;
  int64_t nvalid;
  // fixed split
  const uint32_t* upA;   // [2^nphi]: dense offset of the upper-layer pattern
  const uint32_t* loB;   // [2^nphi * nphi]: offset of the lower-layer pattern per needed residue
  const uint8_t* resid;  // [2^nphi]: sum of occupied orbital indices mod nphi
  // free split: prefix tables of the depth-first rank, [(nel+1) * (2 nphi + 1) * nphi]
  const int64_t* PE;
};

struct blqh_basis {
  blqh_ctx* ctx = nullptr;
  int model = BLQH_MODEL_SPINLESS;  // BLQH_MODEL_SPINFUL: ssector set, only d_id / d_period used
  blqh_sector_spin ssector{};
  blqh_sector_mono msector{};       // BLQH_MODEL_MONOLAYER: only d_id / d_period used
  blqh_sector sector{};
  SectorIdx sx{};
  int64_t dim = 0;
  uint64_t* d_id = nullptr;      // [dim] representatives, ascending
  uint8_t* d_period = nullptr;   // [dim] orbit period (basis::basis_C)
  uint8_t* d_compat = nullptr;   // [dim] 1 if the orbit carries momentum K (phases sum coherently)
  uint32_t* d_map = nullptr;     // [nvalid] state index -> (row << 5) | translation, or ~0u
  // owned index tables
  uint32_t* d_upA = nullptr;
  uint32_t* d_loB = nullptr;
  uint8_t* d_resid = nullptr;
  int64_t* d_PE = nullptr;
};

struct blqh_csr {
  blqh_ctx* ctx = nullptr;
  int64_t dim = 0, nnz = 0;
  int is_complex = 0;
  int precision = BLQH_VAL_FP64;
  int64_t* d_row_ptr = nullptr;  // [dim+1]
  int32_t* d_col = nullptr;      // [nnz]
  void* d_val = nullptr;         // [nnz] double / float, or double2 / float2 when complex
  // FP32 values of the spinless builder: the rest of each FP64 value, FP32(v64 - v32)
  // ([nnz] float, float2 when complex), so that v32 + res carries the FP64
  // element to 2^-48 for the final Rayleigh quotient; null otherwise
  void* d_res = nullptr;
  int lanes_per_row = 32;        // SpMV shape chosen by the tuner
  double mean_row = 0;
  // blocked SpMV (spmv_blocked.cu): per (row block, column tile) slices of 32
  // rows sorted by entry count, stored column-major; blk_state 0 untried,
  // 1 built, -1 not used
  int blk_state = 0;
  int blk_nb = 0, blk_rpb = 0, blk_blocks = 0;
  int64_t blk_steps = 0, blk_slices = 0;
  uint16_t* d_bcol = nullptr;     // [steps][32] column within the tile
  void* d_bval = nullptr;         // [steps][32] float, or float2 when complex
  uint16_t* d_bhdr = nullptr;     // [slices][32] row within the block, 0xFFFF empty
  uint16_t* d_bslen = nullptr;    // [slices] steps of the slice
  int64_t* d_bslice0 = nullptr;   // [blocks * tiles + 1] first slice of (b, t)
  int64_t* d_bstep0 = nullptr;    // [blocks * tiles + 1] first step of (b, t)
  int32_t* d_bsplit = nullptr;    // [blocks * tiles][2 (warps + 1)] warp ranges
  int* d_berr = nullptr;          // set by the kernel when a bounded wait expires
  // dictionary form (real matrices whose off-diagonal values take at most
  // BL_DICT_CAP distinct FP32 values): one 32-bit word per padded entry,
  // column within the 4096-wide tile | value index << 12, the diagonal kept apart
  int blk_dict = 0;               // dictionary size (0: the cols/vals form above)
  int blk_stage = 0;              // dictionary form: bytes of one shared-memory stage (a tile's stream)
  uint32_t* d_bent = nullptr;     // [steps * 32] entries, quad layout per warp range
  float* d_bdict = nullptr;       // [blk_dict] values; index 0 is 0.0f (padding)
  float* d_bdiag = nullptr;       // [dim] diagonal (0 where the row has none)
  int32_t* d_btstart = nullptr;   // [tiles + 1] first column of each tile
  // dictionary form: each (block, tile) stream in chunks ("units") of at most one stage
  int blk_nstage = 0;             // shared-memory stages (2 or 3)
  int64_t blk_units = 0;
  int64_t* d_uchunk0 = nullptr;   // [blocks * tiles + 1] first unit of (b, t)
  int32_t* d_usplit = nullptr;    // [units][2 (warps + 1)] warp ranges within the unit
  int32_t* d_utile = nullptr;     // [units] tile of the unit
  int64_t* d_ustep0 = nullptr;    // [units + 1] first step of the unit
  int64_t* d_uslice0 = nullptr;   // [units + 1] first slice of the unit
};

// Interaction tables and parameters for the row generator (device copy).
struct HamilTables {
  int nphi;
  int is_complex;
  int literal;        // 1: enumerate every translation of the row state (odd nphi)
  double Ec;
  double d, dsas, dv, theta_y;
  const double* V;    // [2][nphi][nphi] (lanczos_hamiltonian.cpp:55-77)
  const double* FTc;  // [2 nphi] cos(2 pi m K / nphi), m = -nphi .. nphi-1
  const double* FTs;  // [2 nphi] sin(...)
  const double* TWc;  // [2 nphi] cos(2 theta_y t / nphi), t = -nphi .. nphi-1
  const double* TWs;
  const double* isq;  // [16][16]: 1 / sqrt(Dl * Dr) for orbit periods Dl, Dr in [1, 16]
};

// Host-side helpers implemented in the .cu files.
// basis.cu: positions of N keys, inserted in this order into a libstdc++
// std::unordered_map<unsigned long, long>, in its iteration order afterwards
// (device array of N owned by the caller).
uint32_t* iteration_positions(blqh_ctx* ctx, const uint64_t* keys, int64_t N);
struct RqPlan;  // hamil.cu: regenerated FP64 Rayleigh quotient of one instance
RqPlan* rq_plan_create(blqh_ctx* ctx, const blqh_basis* B, const blqh_params& p);
int rq_plan_grid(const RqPlan* P);  // block partials the launch writes (2 doubles each)
bool rq_plan_complex(const RqPlan* P);
void rq_plan_launch(blqh_ctx* ctx, RqPlan* P, const double* d_psi, double* d_partial);
int rq_plan_check(blqh_ctx* ctx, RqPlan* P);
void rq_plan_destroy(RqPlan* P);
int hamil_build_impl(blqh_ctx* ctx, const blqh_basis* B, const blqh_params& p, int prec, blqh_csr* M);
void spin_hamil_build_impl(blqh_ctx* ctx, const blqh_basis* B, const blqh_params_spin& p, blqh_csr* M);  // FP64
void mono_hamil_build_impl(blqh_ctx* ctx, const blqh_basis* B, const blqh_params_mono& p, blqh_csr* M);  // FP64
void free_csr(blqh_csr* m);
// observables.cu: pseudospin Sz, Sx and the 2 nphi occupations of a device ground state (spinless).
void observables_impl(blqh_ctx* ctx, const blqh_basis* B, const double* psi, int cplx, double* sz, double* sx,
                      double* occ);
void build_sector_tables(blqh_ctx* ctx, blqh_basis* b);
// spin.cu: ascending bitonic sort of n_pow2 keys (val permuted alongside when not null); padding of
// key[from, to) with ~0; a sorted lookup copy of N keys into skey[n2] (padded) with each key's source index.
void sort_keys_u64(blqh_ctx* ctx, uint64_t* key, uint32_t* val, int64_t n_pow2);
void pad_keys_u64(blqh_ctx* ctx, uint64_t* key, int64_t from, int64_t to);
void sorted_copy_u64(blqh_ctx* ctx, const uint64_t* keys, int64_t N, uint64_t* skey, uint32_t* sidx, int64_t n2);
void coulomb_tables_host(int nphi, int K, const blqh_params& p, double* Ec, std::vector<double>& V);

// Device exclusive scan of n int64 values (in and out may alias).
// Blocked SpMV (spmv_blocked.cu). blocked_mode: BLQH_SPMV_BLOCKED = 0 -> -1
// (never), 1 -> 1 (always), unset -> 0 (the tuner decides).
int blocked_mode();
bool blocked_prepare(blqh_ctx* ctx, blqh_csr* M);
void blocked_release(blqh_csr* M);
void blocked_spmv(blqh_ctx* ctx, const blqh_csr* M, const float2* xs, double* y, const double* bptr,
                  const double* xprev, const int* stop);
int blocked_error(blqh_ctx* ctx, const blqh_csr* M);

void scan_exclusive_i64(blqh_ctx* ctx, const int64_t* in, int64_t* out, int64_t n, int64_t* total_host);
void scan_exclusive_u32_to_i64(blqh_ctx* ctx, const uint32_t* in, int64_t* out, int64_t n, int64_t* total_host);

// tune.cu: shape choices timed once per problem class, cached in a JSON file.
bool tune_enabled();
std::string tune_key(const char* kernel, int prec, int cplx, int64_t dim, double mean_row, int extra);
bool tune_lookup(const std::string& key, int* a, int* b);
void tune_store(const std::string& key, int a, int b, double ms);

// Grid size for a grid-stride kernel: a multiple of the SM count.
int grid_for(blqh_ctx* ctx, int64_t work_items, int block, int per_sm_cap = 32);
// Raises a kernel's dynamic shared-memory limit (a per-kernel, process-wide
// attribute) to at least `bytes`, never lowering it, so that host threads
// preparing launches of different sizes cannot leave it below a size another
// thread is about to launch with.
cudaError_t smem_attr_at_least(const void* func, int bytes);
template <class F>
cudaError_t smem_attr_at_least(F* func, int bytes) {
  return smem_attr_at_least(reinterpret_cast<const void*>(func), bytes);
}
