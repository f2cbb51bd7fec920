/*
 * oracle.h — CPU restatement of thinDB's V2 grouped-aggregation semantics.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the CUDA
 * engine and the timed CPU baseline; nothing in the product links or calls it.
 * thinDB itself is Zig 0.17 and no Zig toolchain exists where this project is
 * built or run, so the reference executor cannot be compiled here; this file
 * restates its semantics from the source and is pinned against the reference's
 * own known-answer tests (tests/golden/).
 *
 * It consumes the same plain-C request and table descriptors as the engine
 * (include/thindb_gpu.h) so a test can hand one request to both.
 */
#ifndef THINDB_ORACLE_H
#define THINDB_ORACLE_H

#include <stdint.h>
#include "../include/thindb_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Run `req` over the host table `t` (t->location must be TGPU_LOC_HOST).
 * threads <= 1: one sequential fold over all rows (the plainest statement).
 * threads  > 1: thinDB's silo shape — scan tiles of 16 row groups staged into
 * 256 hash buckets, each bucket folded by one worker in tile order
 * (src/exec/silo_group_core.zig:11493, :9228, :9348, :7456).
 * Returns a tgpu_status; on TGPU_OK *out holds a result to free. */
int orc_group_by(const tgpu_table_desc *t, const tgpu_request *req, int threads, void **out);

uint64_t orc_result_rows(const void *r);
uint32_t orc_result_cols(const void *r);
uint64_t orc_result_groups(const void *r);      /* groups before HAVING */
uint64_t orc_result_selected(const void *r);    /* rows that passed WHERE */
const void *orc_result_data(const void *r, uint32_t col);
const uint8_t *orc_result_valid(const void *r, uint32_t col); /* one byte per row, 1 = valid */
int orc_result_schema(const void *r, uint32_t col, tgpu_output_column *out);
void orc_result_free(void *r);
const char *orc_last_error(void);

/* Helpers the tests use to pin single conversions. */
double orc_i128_to_f64(uint64_t lo, int64_t hi);
double orc_avg_decimal(uint64_t sum_lo, int64_t sum_hi, uint64_t count, int32_t scale);

#ifdef __cplusplus
}
#endif

#endif
