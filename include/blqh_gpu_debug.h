/* blqh_gpu_debug.h — host-only inspection entry points of libblqh_gpu.so.
 *
 * They run on the CPU (no device needed) and expose internals that the tests
 * check against the oracle. Not part of the reference's interface.
 */
#ifndef BLQH_GPU_DEBUG_H
#define BLQH_GPU_DEBUG_H

#include "blqh_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Dense index of each state among those the reference's depth-first
 * enumeration inserts into basis_set (BLQH_without_spin/basis.cpp:199-259),
 * i.e. its insertion order; -1 for states outside the sector. nvalid_out
 * (optional) receives the number of such states. */
int blqh_debug_sector_index(const blqh_sector* s, int64_t n, const uint64_t* states, int64_t* index_out,
                            int64_t* nvalid_out);

/* Layout the mixed-precision SpMV reads for this matrix: 1 when the
 * blocked copy (row blocks x column tiles, x staged in shared memory) has been
 * built with (2-byte column, FP32 value) entries, 2 when it has been built in
 * dictionary form (4-byte entries: column | index into a shared-memory value
 * table; real matrices with few distinct values), 0 when the row-wise CSR
 * kernels are used; -1 for a null matrix. */
int blqh_debug_spmv_layout(const blqh_csr* M);

#ifdef __cplusplus
}
#endif
#endif
