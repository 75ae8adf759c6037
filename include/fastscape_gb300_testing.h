/*
 * fastscape_gb300_testing.h -- testing hooks of the GB300 FastScape library.
 * They exercise the failure paths on the host side of the boundary; they
 * have no counterpart in the reference (which has no error reporting,
 * fastscape_RB+P.cpp:229-260 uses assert).
 */
#ifndef FASTSCAPE_GB300_TESTING_H
#define FASTSCAPE_GB300_TESTING_H

#include "fastscape_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Installs caller-supplied receiver codes (rings must be FS_NO_FLOW) and runs
 * donors, ordering and accumulation without uplift or erosion. Receivers
 * that contain a cycle make it return FS_ERR_ORDER. */
int fs_test_order_from_receivers(fs_model *m, const int32_t *dir);

/* Runs a device wait on a count that never completes, bounded by `ms`
 * milliseconds; returns FS_ERR_TIMEOUT when the bound works. */
int fs_test_barrier_timeout(fs_model *m, double ms);

/* Selects the receiver kernel: 1 = FP64 reference formula for every cell,
 * 0 (default) = FP32 filter with FP64 fix-up of the cells it cannot decide.
 * Both produce identical receivers. */
int fs_test_set_receiver_path(fs_model *m, int exact);

/* generic = 1: erode with the reference's Newton loop literally (FP64
 * division every iterate, pow(x,1) = x, pow(x,2) = x*x) instead of the
 * unrolled bit-pattern iterates, so that tests can compare the two paths
 * bit for bit. */
int fs_test_set_erosion_path(fs_model *m, int generic);

/* Cells queued for the FP64 fix-up by the receiver filter in the last
 * timestep. */
int fs_test_receiver_fixups(const fs_model *m, int32_t *count);

/* Capacity of the erosion table: drainage counts (cells) below it are
 * covered. The table starts at min(65536, cells+1) records and doubles when
 * a timestep meets a larger count (that timestep is redone, bit-exactly). */
int fs_test_table_capacity(const fs_model *m, int32_t *cap);

#ifdef __cplusplus
}
#endif

#endif
