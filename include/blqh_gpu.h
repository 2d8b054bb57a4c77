/* blqh_gpu.h — C ABI of the GB300 exact-diagonalization library (libblqh_gpu.so).
 *
 * One library call per stage of the reference's exact-diagonalization path
 * (qiongz/BLQH, BLQH_without_spin): sector basis -> Hamiltonian CSR ->
 * Lanczos -> tridiagonal eigensolve -> Ritz vector -> Rayleigh quotient.
 * Every entry point returns an int status (BLQH_OK = 0, negative = error;
 * blqh_last_error() gives the message). Handles own their device memory.
 * Host pointers are plain host memory; nothing here exposes CUDA or torch types.
 * A context is bound to one device and one CUDA stream and is not thread-safe;
 * separate contexts may be used from separate threads.
 *
 * Each declaration names the reference interface it replaces (file:line,
 * within the reference project).
 */
#ifndef BLQH_GPU_H
#define BLQH_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BLQH_OK 0
#define BLQH_ERR_ARG -1         /* invalid argument */
#define BLQH_ERR_CUDA -2        /* CUDA runtime error (message has details) */
#define BLQH_ERR_NOMEM -3       /* device allocation failed */
#define BLQH_ERR_UNSUPPORTED -4 /* sector or option outside what the library implements */
#define BLQH_ERR_CAPACITY -5    /* a per-row buffer overflowed (reported, never written past) */
#define BLQH_ERR_STATE -6       /* call out of order (e.g. Ritz vector before iterate) */
#define BLQH_ERR_TIMEOUT -7     /* a bounded device wait gave up */

/* Representative convention of the sector basis. */
#define BLQH_REP_REFERENCE 0 /* survivor of the reference's unordered_map orbit filter (basis.cpp:82-99) */
#define BLQH_REP_MIN 1       /* numerically smallest member of each orbit */

/* Precision of the stored CSR values. Products always accumulate in FP64. */
#define BLQH_VAL_FP64 0
#define BLQH_VAL_FP32 1

typedef struct blqh_ctx blqh_ctx;
typedef struct blqh_basis blqh_basis;
typedef struct blqh_csr blqh_csr;
typedef struct blqh_lanczos blqh_lanczos;

/* Sector of the spinless bilayer (BLQH_without_spin/basis.h:25-56):
 * nphi orbitals per layer, nel electrons, nel_up of them in the upper layer
 * (nel_up < 0: free layer split, basis.cpp:240-259), total momentum J
 * (J < 0: no filter) and translation sector K (K < 0: no translation symmetry). */
typedef struct {
  int nphi, nel, nel_up, J, K;
  int rep_mode; /* BLQH_REP_* */
} blqh_sector;

/* Model parameters of lhamil::set_hamil (BLQH_without_spin/lanczos_hamiltonian.h:51):
 * torus lengths lx, ly; Landau level nLL; layer distance d; tunnelling
 * Delta_SAS; bias Delta_V; twist phases theta_x, theta_y. */
typedef struct {
  double lx, ly, d, delta_sas, delta_v, theta_x, theta_y;
  int nLL;
} blqh_params;

/* Sector of the spinful bilayer (BLQH_with_spin/basis.h:35, basis::init(nphi, nel, nel_up, nel_su, J, K)):
 * 4 blocks of nphi orbitals (upper layer spin up, upper down, lower up, lower down); nel_up electrons
 * in the upper layer (< 0: free split), nel_su with spin up (< 0: any). 4 * nphi <= 60. */
typedef struct {
  int nphi, nel, nel_up, nel_su, J, K;
  int rep_mode; /* BLQH_REP_* */
} blqh_sector_spin;

/* Model parameters of the spinful lhamil::set_hamil (BLQH_with_spin/lanczos_hamiltonian.h:52):
 * as blqh_params plus the Zeeman splitting delta_z and the parallel-field phase theta_b. */
typedef struct {
  double lx, ly, d, delta_sas, delta_v, delta_z, theta_b, theta_x, theta_y;
  int nLL;
} blqh_params_spin;

/* Sector of the monolayer (Monolayer/basis.h:21-53, basis::init(nphi, nel, J, K)): nphi orbitals,
 * nel electrons, total momentum J (J < 0: no filter) and translation sector K in [0, C), where
 * C = gcd(nel, nphi) translations move every electron by nphi / C orbitals (K < 0: no translation
 * symmetry). 2 <= nphi <= 31 (the reference's enumeration holds a state in an int,
 * Monolayer/basis.cpp:218-220). */
typedef struct {
  int nphi, nel, J, K;
  int rep_mode; /* BLQH_REP_* */
} blqh_sector_mono;

/* Model parameters of the monolayer lhamil::set_hamil(sector, lx, ly, nphi, nLL)
 * (Monolayer/lanczos_hamiltonian.h:45): torus lengths lx, ly and Landau level nLL. */
typedef struct {
  double lx, ly;
  int nLL;
} blqh_params_mono;

/* Lanczos options. */
typedef struct {
  int max_steps;      /* lambda: upper bound on Krylov steps (lanczos_hamiltonian.h:15) */
  int reorth;         /* 1: full FP64 reorthogonalization (three-term step, then one classical Gram-Schmidt
                         pass against every stored vector); 0: plain three-term recurrence */
  double tol;         /* stop when the lowest Ritz value moves less than tol between checks (0: run max_steps) */
  int check_every;    /* steps between convergence checks (>= 1) */
  uint64_t seed;      /* start-vector seed */
  int rng;            /* start vector: 0 = std::mt19937 stream as matrix.cpp:54-75 (host);
                         1 = mt19937-64 genrand64_real3 (host); 2 = counter-based generator on
                         the device (splitmix64 of seed and index), no host work */
  int accumulate;     /* SpMV with FP32 values: 0 = double-float accumulation (FP32 pairs with error-free
                         transformations, ~2^-48 per product; keeps the per-nonzero work off GB300's
                         slow FP64 pipe); 1 = native FP64 FMA. FP64 values always use native FP64. */
} blqh_lanczos_opts;

/* ---- context ------------------------------------------------------------ */
int blqh_ctx_create(int device, blqh_ctx** out);
int blqh_ctx_destroy(blqh_ctx* ctx);
const char* blqh_last_error(const blqh_ctx* ctx); /* ctx may be NULL: last error of this thread */
int blqh_ctx_synchronize(blqh_ctx* ctx);
/* Kernel launches and, when enabled (enable = 1; -1 keeps the setting), device time (ms)
 * per kernel class since the last reset: 0 = SpMV, 1 = Lanczos vector updates and
 * reorthogonalization, 2 = CSR build and FP64 Rayleigh regeneration, 3 = basis,
 * 4 = everything else (eigensolver, Ritz vector, scans, start vector). Arrays of 5. */
int blqh_ctx_timers(blqh_ctx* ctx, int enable, double* ms_out5, int64_t* launches_out5);
int blqh_ctx_reset_timers(blqh_ctx* ctx);
/* Event markers on the context's stream: record marker slot (0..7); elapsed device time
 * between two recorded markers (waits for the later one). */
int blqh_ctx_mark(blqh_ctx* ctx, int slot);
int blqh_ctx_elapsed_ms(blqh_ctx* ctx, int slot_from, int slot_to, double* ms);

/* ---- sector basis (replaces basis::init, BLQH_without_spin/basis.cpp:61-119) ---- */
int blqh_basis_build(blqh_ctx* ctx, const blqh_sector* sector, blqh_basis** out);
int blqh_basis_size(const blqh_basis* b, int64_t* dim);
/* host copies of basis::id (sorted representatives) and basis::basis_C (orbit periods) */
int blqh_basis_get(blqh_ctx* ctx, const blqh_basis* b, uint64_t* ids, int16_t* periods);
int blqh_basis_destroy(blqh_basis* b);

/* Spinful basis (replaces BLQH_with_spin basis::init / generate_fixed_density / generate_all_density,
 * basis.cpp:74-141, 240-300, with the same representative survivor; translations act on all four
 * blocks, basis.cpp:401-477). The handle works with blqh_basis_size/get/destroy. */
int blqh_basis_build_spin(blqh_ctx* ctx, const blqh_sector_spin* sector, blqh_basis** out);

/* ---- Hamiltonian (replaces lhamil::set_hamil / peer_set_hamil, lanczos_hamiltonian.cpp:87-385) ---- */
/* value_precision: BLQH_VAL_FP64 or BLQH_VAL_FP32 (stored values; FP64 accumulation) */
int blqh_hamil_build(blqh_ctx* ctx, const blqh_basis* b, const blqh_params* p, int value_precision,
                     blqh_csr** out);
/* Spinful Hamiltonian (replaces BLQH_with_spin lhamil::peer_set_hamil, lanczos_hamiltonian.cpp:86-927):
 * FP64 values; one thread block per row, the row in a shared-memory table sized by the number of moves
 * from a state (no limit on the sector's size; BLQH_ERR_UNSUPPORTED when the table for that many
 * electrons would not fit in shared memory). */
int blqh_hamil_build_spin(blqh_ctx* ctx, const blqh_basis* b, const blqh_params_spin* p, blqh_csr** out);
/* The same with a choice of stored value precision (BLQH_VAL_FP64, or BLQH_VAL_FP32: the FP64 sums rounded
 * once); with FP32 values finish the energy with blqh_lanczos_rayleigh_fp64_spin. */
int blqh_hamil_build_spin_prec(blqh_ctx* ctx, const blqh_basis* b, const blqh_params_spin* p, int value_precision,
                               blqh_csr** out);

/* Monolayer basis (replaces Monolayer basis::init / generate, basis.cpp:59-119, 216-235, with the same
 * representative survivor). The handle works with blqh_basis_size/get/destroy; periods are basis_C. */
int blqh_basis_build_mono(blqh_ctx* ctx, const blqh_sector_mono* sector, blqh_basis** out);
/* Monolayer Hamiltonian (replaces Monolayer lhamil::set_hamil, lanczos_hamiltonian.cpp:77-198, and the
 * dense hamil::set_hamil, hamiltonian.cpp:29-103, which generates the same elements): FP64 values,
 * complex unless K <= 0 or 2 K == C. One warp per row; the row is accumulated in the reference's
 * order, so values equal the reference's sums term by term. */
int blqh_hamil_build_mono(blqh_ctx* ctx, const blqh_basis* b, const blqh_params_mono* p, blqh_csr** out);
/* Classical energy E_cl of the monolayer Hamiltonian's diagonal (lanczos_hamiltonian.cpp:68-74): the
 * reference integrates integral_1^inf t^-1/2 e^-zt dt numerically (GSL qagiu, matrix.cpp:320-336);
 * here it is sqrt(pi / z) erfc(sqrt(z)), the same integral in closed form. Host only. */
int blqh_mono_classical_energy(int nphi, double lx, double ly, double* e_cl);
/* Interaction table of the monolayer (lhamil::init_Coulomb_matrix, lanczos_hamiltonian.cpp:58-67):
 * V[s * nphi + q_y] for s, q_y in [0, nphi), host only; V holds nphi * nphi doubles. */
int blqh_mono_coulomb_table(int nphi, double lx, double ly, int nLL, double* V);
int blqh_csr_info(const blqh_csr* m, int64_t* dim, int64_t* nnz, int* is_complex, int* value_precision);
/* Host copy: row_ptr[dim+1], col[nnz], val[nnz] (real) or val[2*nnz] (re, im interleaved), as doubles. */
int blqh_csr_get(blqh_ctx* ctx, const blqh_csr* m, int64_t* row_ptr, int32_t* col, double* val);
int blqh_csr_destroy(blqh_csr* m);
/* y = H x with host buffers (Mat::operator*, matrix.cpp:244-267); length dim, or 2*dim interleaved if complex */
int blqh_spmv(blqh_ctx* ctx, const blqh_csr* m, const double* x, double* y);

/* ---- Lanczos (replaces lhamil::coeff_explicit_update, diag, eigenstates_reconstruction,
 *      ground_state_energy: lanczos_hamiltonian.cpp:453-656) ---- */
int blqh_lanczos_create(blqh_ctx* ctx, const blqh_csr* m, const blqh_lanczos_opts* opts, blqh_lanczos** out);
/* Optional start vector from the host (length dim, or 2*dim interleaved if complex); normalized by the library. */
int blqh_lanczos_set_start(blqh_lanczos* l, const double* x);
/* Pass 1: run the recurrence until convergence, breakdown or max_steps. */
int blqh_lanczos_iterate(blqh_lanczos* l, int* steps_done);
/* alpha[steps], beta[steps+1] (beta[0] = 1, beta[j] couples steps j-1 and j, as lhamil::norm) */
int blqh_lanczos_coeffs(blqh_lanczos* l, double* alpha, double* beta);
/* Tridiagonal eigensolve on the device (replaces diag_dsyevd, matrix.cpp:288-305):
 * all Ritz values ascending (eigenvalues[steps]) and the ground Ritz vector in the Krylov basis (psi0[steps]).
 * Either pointer may be NULL. */
int blqh_lanczos_eig(blqh_lanczos* l, double* eigenvalues, double* psi0);
/* Ground state in the sector basis, sum_l psi0[l] v_l, normalized (kept on the device; copied out if psi != NULL). */
int blqh_lanczos_ritz_vector(blqh_lanczos* l, double* psi);
/* <psi|H|psi> with the ground state from blqh_lanczos_ritz_vector, using the stored CSR values. */
int blqh_lanczos_rayleigh(blqh_lanczos* l, double* energy);
/* <psi|H|psi> with FP64-class matrix elements: the mixed-precision finisher. For an FP32 matrix from
 * blqh_hamil_build the elements are its FP32 values plus the FP32 rests of the FP64 values the builder
 * computed (stored with the matrix; (basis, params) are then only checked against it); otherwise, or
 * with BLQH_RQ_REGEN=1, they are regenerated in FP64 from (basis, params). Replaces the reference's
 * final Rayleigh quotient (lanczos_hamiltonian.cpp:646-656) for FP32-valued runs. */
int blqh_lanczos_rayleigh_fp64(blqh_lanczos* l, const blqh_basis* b, const blqh_params* p, double* energy);
/* The energy the reference prints: its eigenstates_reconstruction forms psir_0 = sum_l psi_0[l] conj(phi_l)
 * (lanczos_hamiltonian.cpp:610-644, the conjugation at :625, :632) and ground_state_energy returns
 * <psir_0|H|psir_0> (:646-656), i.e. <conj(psi)|H|conj(psi)> for the ground state psi. That equals the
 * ground energy in real sectors only; in complex sectors it is the expectation of conj(H). This entry point
 * reproduces it from the library's ground state: with b and p (both non-NULL) from FP64 matrix elements
 * regenerated on the fly, else from the stored CSR values. */
int blqh_lanczos_rayleigh_conj(blqh_lanczos* l, const blqh_basis* b, const blqh_params* p, double* energy);
/* Ground-state observables after blqh_lanczos_ritz_vector, as the reference evaluates them from psir_0
 * (lanczos_hamiltonian.cpp:658-736; spinless): pseudospin_Sz, pseudospin_Sx and the occupation numbers
 * occ[2 * nphi] (upper layer orbitals 0..nphi-1, then the lower layer). Any output may be NULL. */
int blqh_lanczos_observables(blqh_lanczos* l, const blqh_basis* b, double* sz, double* sx, double* occ);
/* Spinful ground_state_energy (BLQH_with_spin/lanczos_hamiltonian.cpp:1192-1215) with the matrix elements
 * regenerated in FP64 by the row generator, nothing stored: the mixed-precision finisher. */
int blqh_lanczos_rayleigh_fp64_spin(blqh_lanczos* l, const blqh_basis* b, const blqh_params_spin* p,
                                    double* energy);
/* The spinful model's ground-state observables after blqh_lanczos_ritz_vector (replaces Sz, pseudospin_Sz,
 * upper_Sz, down_Sz, pseudospin_Sx, spinflip_tunneling and occupatation_number of BLQH_with_spin/
 * lanczos_hamiltonian.cpp:1217-1593, which the reference evaluates from its conjugated psir_0): out[0..5] =
 * Sz, pseudospin_Sz, upper_Sz, down_Sz, pseudospin_Sx, spinflip_tunneling; out[6 .. 6 + 2 nphi) = the
 * occupation numbers (alpha 0: block 0 orbitals, then alpha 1: block 1). */
int blqh_lanczos_observables_spin(blqh_lanczos* l, const blqh_basis* b, double* out);
int blqh_lanczos_destroy(blqh_lanczos* l);

/* ---- one-call ground state: basis -> CSR -> Lanczos -> Rayleigh quotient ----
 * The whole path of the reference main (BLQH_without_spin/main.cpp:34-41) for one sector.
 * energy = final E_gs; steps = Krylov steps used; psi (optional, host) = ground state. */
typedef struct {
  double energy;     /* E_gs: FP64 Rayleigh quotient of the ground Ritz vector */
  double ritz0;      /* lowest Ritz value of the Krylov tridiagonal */
  int steps;         /* Krylov steps */
  int64_t dim, nnz;
} blqh_result;
int blqh_ground_state(blqh_ctx* ctx, const blqh_sector* s, const blqh_params* p, int value_precision,
                      const blqh_lanczos_opts* opts, const double* start, double* psi, blqh_result* out);

/* ---- batched sweep: many (sector, parameter point) instances in one persistent launch ----
 * Replaces the sweep loops the reference keeps in its drivers (BLQH_without_spin/main.cpp:77-115,
 * 134-181): every instance gets its basis (shared between instances of the same sector), its CSR
 * and a Krylov space; one persistent kernel then runs all instances' Lanczos recurrences, one
 * instance per thread block at a time, taken from a device work queue in decreasing cost, with
 * full FP64 reorthogonalization and the tridiagonal ground state computed inside the block.
 * Mixed precision (value_precision = BLQH_VAL_FP32) finishes each energy with the FP64
 * regenerated Rayleigh quotient; FP64 values finish with the stored CSR. */
#define BLQH_MODEL_SPINLESS 0
#define BLQH_MODEL_SPINFUL 1
#define BLQH_MODEL_MONOLAYER 2
typedef struct {
  int model;            /* BLQH_MODEL_SPINLESS: sector, params; BLQH_MODEL_SPINFUL: ssector, sparams;
                           BLQH_MODEL_MONOLAYER: msector, mparams (spinful and monolayer instances keep
                           FP64 values and finish with them) */
  blqh_sector sector;
  blqh_params params;
  blqh_sector_spin ssector;
  blqh_params_spin sparams;
  blqh_sector_mono msector;
  blqh_params_mono mparams;
} blqh_instance;

typedef struct {
  int lambda;           /* Lanczos steps per instance (fewer when the Krylov space is exhausted) */
  int value_precision;  /* BLQH_VAL_FP32 or BLQH_VAL_FP64 */
  uint64_t seed;        /* start vectors: splitmix64 of (seed, instance number, index) */
  int threads;          /* threads per block: 0 = default (256), else 256 or 512 */
  int lanes_per_row;    /* SpMV lanes per row: 0 = from the mean row length, else 4, 8, 16 or 32 */
  int use_graph;        /* 1: capture the solve in a CUDA graph on the first call, replay it afterwards */
} blqh_batch_opts;

typedef struct {
  double energy;        /* finished E_gs (see above) */
  double ritz0;         /* lowest Ritz value of the instance's tridiagonal */
  double resid;         /* beta_m |y_m|: residual norm of the Ritz pair */
  int64_t dim, nnz;
  int steps;            /* Krylov steps run */
  int second_passes;    /* steps whose full Gram-Schmidt pass had to be repeated (DGKS criterion) */
} blqh_batch_result;

typedef struct blqh_batch blqh_batch;
/* Bases, CSRs and Krylov storage for n instances (device memory for all of them at once). */
int blqh_batch_create(blqh_ctx* ctx, const blqh_instance* inst, int n, const blqh_batch_opts* opts,
                      blqh_batch** out);
/* Run every instance's Lanczos and finisher (asynchronous launches, one synchronize at the end). */
int blqh_batch_solve(blqh_batch* b);
int blqh_batch_results(const blqh_batch* b, blqh_batch_result* out);
/* Host copy of instance i's ground state (dim doubles, or 2*dim interleaved if complex). */
int blqh_batch_ground_state(const blqh_batch* b, int i, double* psi);
/* Shape the solve used: threads per block, lanes per row, blocks per SM. */
int blqh_batch_shape(const blqh_batch* b, int* threads, int* lanes_per_row, int* blocks_per_sm);
/* Device time of the last solve: the persistent Lanczos launch and the finishers after it (ms,
 * CUDA events on the context stream), and the number of kernel launches one solve makes. */
int blqh_batch_timing(const blqh_batch* b, double* lanczos_ms, double* finish_ms, int* launches);
int blqh_batch_destroy(blqh_batch* b);
/* create + solve + results + destroy */
int blqh_batch_run(blqh_ctx* ctx, const blqh_instance* inst, int n, const blqh_batch_opts* opts,
                   blqh_batch_result* out);

/* ---- learned start vector (no counterpart in the reference, whose start is random:
 *      Vec::init_random, matrix.cpp:54-75) ----
 * A multilayer perceptron: input = the 2*nphi occupation bits of a basis state (as +-1) and the
 * parameter point (d/l, Delta_SAS); 3 hidden layers of `width` units with tanh; one real output,
 * the state's amplitude. BF16 weights and activations, FP32 accumulation on the tensor cores
 * (tcgen05 with TMA loads and tensor-memory accumulators for widths that are multiples of 32 up
 * to 256, mma.sync otherwise or with BLQH_MLP_TC=0); FP32 master weights updated by Adam. Training minimizes, per parameter point, one minus the
 * squared overlap of the prediction with the target ground state. Real sectors only. */
typedef struct blqh_mlp blqh_mlp;
int blqh_mlp_create(blqh_ctx* ctx, int n_bits, int width, uint64_t seed, blqh_mlp** out);
int blqh_mlp_num_params(const blqh_mlp* m, int64_t* n);
/* Flat FP32 parameters: Wt0 [width][K0] | b0 [width] | Wt1 [width][width] | b1 | Wt2 [width][width] | b2 |
 * w3 [width] | b3 [1], K0 = n_bits + 2 rounded up to 32; Wt[n][k] weighs input k into unit n. */
int blqh_mlp_get_params(const blqh_mlp* m, float* params);
int blqh_mlp_set_params(blqh_mlp* m, const float* params);
/* Normalized prediction over the basis for one parameter point (host output, dim doubles). */
int blqh_mlp_predict(blqh_mlp* m, const blqh_basis* b, double d, double delta_sas, double* psi);
/* Mean loss and its gradient (host, num_params floats) over npts points: cond[2*npts] = (d, Delta_SAS),
 * targets[npts * dim] (host, any norm and sign). No update. */
int blqh_mlp_loss_grad(blqh_mlp* m, const blqh_basis* b, int npts, const double* cond, const double* targets,
                       double* loss, float* grad);
/* `steps` full-batch Adam steps (learning rate lr) over the npts points; loss_out[steps] (optional). */
int blqh_mlp_train(blqh_mlp* m, const blqh_basis* b, int npts, const double* cond, const double* targets, int steps,
                   double lr, double* loss_out);
int blqh_mlp_destroy(blqh_mlp* m);

/* ---- SpMV without any device allocation ----
 * No counterpart in the reference. For callers that cannot call cudaMalloc (their
 * device memory comes from a host framework's pool, or allocating would stall
 * their streams): y = H x for a real CSR matrix with FP32 values, accumulated in
 * double-float, all pointers device memory owned by the caller; the only scratch
 * (x split into FP32 pairs) is a built-in array of BLQH_NOALLOC_MAX_DIM entries
 * (8 MiB per GPU, kept until exit). dim above that is rejected with
 * BLQH_ERR_ARG. The call is asynchronous on `stream` (NULL: the default stream).
 * The first call on a device looks up the array's address; make it before any
 * stream capture. The address is cached per device number and is stale after a
 * cudaDeviceReset of that device. Calls share the array, which keeps the last
 * call's contents: calls that overlap on the GPU race, so order them. */
#define BLQH_NOALLOC_MAX_DIM (1 << 20)
int blqh_spmv_f32_noalloc(const int64_t* row_ptr, const int32_t* col, const float* val, int64_t dim,
                          const double* x, double* y, void* stream);

/* ---- host utilities (not hot) ---- */
/* Start vector as the reference draws it (lanczos_hamiltonian.cpp:468-483): rng 0 = std::mt19937,
 * rng 1 = mt19937-64 genrand64_real3 (the reference's pre-C++11 branch). complex: 2*dim doubles. */
int blqh_start_vector(uint64_t seed, int rng, int64_t dim, int is_complex, double* out);

#ifdef __cplusplus
}
#endif
#endif /* BLQH_GPU_H */
