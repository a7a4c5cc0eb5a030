/*
 * CPU oracle for the GB300 wavelet-tree path — TEST INFRASTRUCTURE ONLY.
 *
 * A plain C++ restatement of mfranzreb/ECL_wavelet's levelwise wavelet tree,
 * its BitArray layout and RankSelect support, plus plain-scan answers
 * (access = text[i], rank = count before i, select = position of k-th).
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load this library; the product path never does.
 *
 * Parity pinning: this restatement is checked against the known-answer
 * vectors of the reference's own test suite (tests/test_wavelet_tree.cu,
 * tests/test_rank_select.cu), restated as closed-form fixtures in
 * tests/golden/.  Each function in ewt_oracle.cpp cites the reference
 * file:line it follows.
 */
#ifndef EWT_ORACLE_H
#define EWT_ORACLE_H
#include <stdint.h>

#include "ewt.h" /* shared export ids and ewt_info */

#ifdef __cplusplus
extern "C" {
#endif

/* Tree build from a host text of elem_size-byte unsigned symbols.  alphabet
 * (sorted, as uint64) may be NULL with sigma = 0 to request detection. */
int ewto_build(const void* data, uint64_t n, int elem_size,
               const uint64_t* alphabet, uint64_t sigma, void** out);
void ewto_free(void* h);
/* The same tree built on nthreads host threads (<= 0: all OpenMP threads)
 * without keeping the text: the CPU baseline and the full-size checker.
 * Exports and the walk queries work as for ewto_build; the plain-scan
 * calls return EWT_ERR_UNSUPPORTED (use ewto_scan_batch). */
int ewto_build_mt(const void* data, uint64_t n, int elem_size,
                  const uint64_t* alphabet, uint64_t sigma, int nthreads,
                  void** out);
/* Plain-scan answers of a mixed batch (types 0/1/2) straight from a 1- or
 * 2-byte text over the minimal alphabet [0, sigma), in O(n + m log m):
 * access = text[i] (0 past the end), rank = occurrences before i (i <= n),
 * select = position of the k-th occurrence (n when fewer); invalid queries
 * give UINT64_MAX and EWT_ERR_QUERY. */
int ewto_scan_batch(const void* text, uint64_t n, int elem_size,
                    uint64_t sigma, const uint8_t* types, const uint64_t* idx,
                    const uint64_t* sym, uint64_t m, uint64_t* out,
                    int nthreads);
int ewto_info(void* h, ewt_info* info);
int ewto_export(void* h, int component, int level, void* buf,
                uint64_t cap_bytes, uint64_t* size_bytes);

/* Queries by walking the structure (restating the reference's device walk).
 * Symbols are given in the ORIGINAL alphabet and remapped by lower_bound, as
 * the reference's host API does.  nthreads <= 0 uses all OpenMP threads. */
int ewto_access(void* h, const uint64_t* idx, uint64_t m, uint64_t* out,
                int nthreads);
int ewto_rank(void* h, const uint64_t* idx, const uint64_t* sym, uint64_t m,
              uint64_t* out, int nthreads);
int ewto_select(void* h, const uint64_t* k, const uint64_t* sym, uint64_t m,
                uint64_t* out, int nthreads);
/* Mixed batch: types 0 = access, 1 = rank, 2 = select. */
int ewto_mixed(void* h, const uint8_t* types, const uint64_t* idx,
               const uint64_t* sym, uint64_t m, uint64_t* out, int nthreads);

/* Plain-scan answers straight from the stored text (no tree involved). */
int ewto_scan_access(void* h, const uint64_t* idx, uint64_t m, uint64_t* out);
int ewto_scan_rank(void* h, const uint64_t* idx, const uint64_t* sym,
                   uint64_t m, uint64_t* out);
int ewto_scan_select(void* h, const uint64_t* k, const uint64_t* sym,
                     uint64_t m, uint64_t* out);

/* Standalone RankSelect over caller-given bit arrays.  words holds, for each
 * array in turn, ceil(bits[a]/32) packed LSB-first words. */
int ewto_rs_build(const uint32_t* words, const uint64_t* bits,
                  uint32_t num_arrays, void** out);
void ewto_rs_free(void* h);
int ewto_rs_export(void* h, int component, int array, void* buf,
                   uint64_t cap_bytes, uint64_t* size_bytes);
uint64_t ewto_rs_rank(void* h, int array, uint64_t pos, int value);
uint64_t ewto_rs_select(void* h, int array, uint64_t i, int value);
void ewto_rs_rank_batch(void* h, int array, const uint64_t* pos, uint64_t m,
                        int value, uint64_t* out, int nthreads);
void ewto_rs_select_batch(void* h, int array, const uint64_t* idx, uint64_t m,
                          int value, uint64_t* out, int nthreads);

/* Alphabet-shape helpers used by the known-answer tests. */
int ewto_minimal_codes(uint64_t sigma, uint64_t* lens, uint64_t* codes,
                       uint64_t cap, uint64_t* count);
int ewto_node_infos(uint64_t sigma, uint64_t* starts, uint64_t* levels,
                    uint64_t cap, uint64_t* count);
uint64_t ewto_node_pos(uint64_t sigma, uint64_t symbol, uint32_t level);
uint64_t ewto_prev_pow2(uint64_t n);
uint32_t ewto_ceil_log2(uint64_t n);
int ewto_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
