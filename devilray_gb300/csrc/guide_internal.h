// guide_internal.h -- the guiding network's launchers for the renderer.
#pragma once

#include "dr_internal.h"

namespace dr {

// Network outputs y[slot][40] for the rows list[0 .. *count) (positions and
// directions read at the same slots). At most max_rows rows. With `decoded`,
// each row's mixture is stored decoded for the shading kernel instead
// (guide_store_decoded).
cudaError_t launch_guide_infer(const dr_guide *g, const float *pos, const float *dir, const uint32_t *list,
                               const uint32_t *count, uint32_t max_rows, float *y, cudaStream_t st,
                               bool decoded = false);

// Adam steps the network has taken (enqueued).
uint32_t guide_steps(const dr_guide *g);

// One Adam step on rows [0, n) of the given arrays.
dr_status guide_train_step(dr_guide *g, const float *pos, const float *dir, const float *sdir, const float *weight,
                           uint32_t n, cudaStream_t st);

}  // namespace dr
