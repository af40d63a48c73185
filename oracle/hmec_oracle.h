/*
 * hmec_oracle.h -- CPU restatement of the H-MEC per-timestep hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the oracle the GPU library is compared
 * against (tests, __graft_entry__.smoke, and the CPU-baseline leg of
 * bench.py).  Nothing in the product links or calls it.
 *
 * It restates cpp/h_mec_rsf_v9.cpp:118-159 (helpers), :376-1726 (one
 * timestep) and cpp/constants.hpp:13-146 (constants) in plain C with
 * column-major grids laid out like Eigen's MatrixXd.  Every section is a
 * separate function so tests can replay one section on a given state.
 *
 * Parity status: the reference publishes no golden vectors, known-answer
 * tests or fixtures, and it cannot be built here (Eigen, HDF5, MKL/Pardiso
 * and icpc are absent), so this restatement is pinned by hand-derived
 * known answers (tests/test_oracle_pins.py) and by the reference's own
 * printed check values (nucleation size and cohesive zone, :363-370).
 *
 * The sparse direct solve that the reference hands to Pardiso (:1050-1052)
 * is a callback: the Python driver supplies SciPy SuperLU with iterative
 * refinement.
 */
#ifndef HMEC_ORACLE_H
#define HMEC_ORACLE_H

#include <stdint.h>
#include "../include/hmec.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct hmo_state hmo_state;

/* Solve A x = b for the CSR matrix (duplicates already summed). Return 0 on success. */
typedef int (*hmo_solve_fn)(void* user, int32_t n, const int64_t* indptr, const int32_t* indices,
                            const double* data, const double* rhs, double* x);

void hmo_params_default(hmec_params* p);
hmo_state* hmo_create(const hmec_params* p);
void hmo_destroy(hmo_state* st);

int64_t hmo_marknum(const hmo_state* st);
int32_t hmo_unknowns(const hmo_state* st);
double* hmo_field(hmo_state* st, int32_t field);   /* column-major storage */
double* hmo_marker(hmo_state* st, int32_t field);
double hmo_get_scalar(const hmo_state* st, int32_t id);
void hmo_set_scalar(hmo_state* st, int32_t id, double v);
/* Eigen LinSpaced coordinates: which = 0 x, 1 y, 2 xvx, 3 yvx, 4 xvy, 5 yvy, 6 xp, 7 yp */
const double* hmo_coords(const hmo_state* st, int32_t which);

/* Sections, in the order main() runs them. */
void hmo_markers_to_nodes(hmo_state* st);                       /* :376-583 */
/* Threads of the marker loop of hmo_markers_to_nodes (default 1, the serial
 * loop in marker order).  n > 1: contiguous marker shares summed per thread
 * and added in thread order -- the reference's OpenMP loop (:384) without
 * its unsynchronised additions; equal to the serial loop up to rounding. */
void hmo_set_threads(hmo_state* st, int32_t n);
void hmo_timestep_begin(hmo_state* st);                         /* :585-608 */
void hmo_iter_prepare(hmo_state* st);                           /* :611-677 */
/* :682-1049 -- builds R and the CSR of L; returns nnz. */
int64_t hmo_assemble(hmo_state* st);
void hmo_csr(const hmo_state* st, const int64_t** indptr, const int32_t** indices, const double** data,
             const double** rhs);
/* :1060-1456 given the solution S; returns 1 when the exit test passed. */
int32_t hmo_iter_finish(hmo_state* st, const double* S);
/* A whole global iteration (prepare, assemble, solve, finish); returns stop flag or <0 on solve error. */
int32_t hmo_global_iteration(hmo_state* st, hmo_solve_fn solve, void* user);
void hmo_timestep_end(hmo_state* st);                           /* :1463-1559, :1658-1726 */
void hmo_advect_markers(hmo_state* st);                         /* :1561-1656 (enabled form) */
/* :377-1726 -- returns number of global iterations or <0 on solve error. */
int32_t hmo_timestep(hmo_state* st, hmo_solve_fn solve, void* user);

/* Last global iteration's bookkeeping. */
int32_t hmo_last_ynpl(const hmo_state* st);
double hmo_last_dsylsq(const hmo_state* st);
int32_t hmo_rsf_noconv(const hmo_state* st);

#ifdef __cplusplus
}
#endif
#endif
