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

/* One convolution of the learned surrogate's kernels on host buffers (the
 * library allocates, copies, runs on the current device and copies back),
 * for checking the tensor-core kernels against a CPU convolution. Tensors
 * are NHWC BF16 (uint16 bit patterns), B images of H x W pixels; weights
 * are BF16 [cout][taps][cin] with tap = 3*dy + dx (taps 9: 3x3 with zero
 * padding; taps 1: 1x1); cin and cout multiples of 16.
 *   mode 0 (forward):  out[p][co] = act(bias[co] + sum x[p+off][ci] w[co][tap][ci])
 *                      x: [B,H,W,cin], out: [B,H,W,cout] BF16; act = ReLU when
 *                      relu, bias may be NULL; mask NULL.
 *   mode 1 (data gradient): out[p][ci] = sum dy[p-off][co] w[co][tap][ci],
 *                      zeroed where mask[p][ci] <= 0 (mask may be NULL);
 *                      x holds dy [B,H,W,cout], out: [B,H,W,cin] BF16.
 *   mode 2 (weight gradient): out[co][tap][ci] = sum_p dy[p][co] x[p+off][ci]
 *                      (FP32); x: [B,H,W,cin], w holds dy [B,H,W,cout].
 *   mode 3: mode 0 with the output written as planes of a wider tensor (two
 *                      sentinel planes on each side, which must stay
 *                      untouched: FS_ERR_CUDA otherwise); out as in mode 0.
 *   mode 4: mode 3 with the output upsampled 2x (nearest) as it is stored:
 *                      out [B,2H,2W,cout].
 * No counterpart in the reference (it has no learned part). */
int fs_test_sg_conv(int mode, int B, int H, int W, int cin, int cout, int taps,
                    const uint16_t *x, const uint16_t *w, const float *bias, int relu,
                    const uint16_t *mask, void *out);

#ifdef __cplusplus
}
#endif

#endif
