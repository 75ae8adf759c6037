// sg_net.h -- shared between the surrogate network (sg_net.cu) and the
// judged ensemble (sg_ensemble.cu). Not part of the public ABI.
#pragma once

#include "fastscape_gb300.h"
#include "fastscape_surrogate.h"
#include "sg_ops.h"

namespace sg {

// Per-sample constants for a jump of `jump` timesteps of length dt from a
// field whose maximum is hmax, towards a field whose maximum is hmax_next
// (the loss weight (u / max(hmax_next, u))^2; pass hmax when unknown).
SampleMeta make_meta(const fs_params &p, double hmax, double hmax_next, int jump, double dt);

}  // namespace sg

// Jumps n device fields hin[k] with constants p[k] and drainage counts
// cnt[k] into hout[k] (hout[k] may be hin[k]); returns when they are written.
int sg_predict_fields(fs_surrogate *s, int n, double *const *hin, double *const *hout,
                      const fs_params *p, uint32_t *const *cnt);
