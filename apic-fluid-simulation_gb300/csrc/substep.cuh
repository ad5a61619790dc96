// substep.cuh — the substep loop's device-side control (src/apic.rs:2429-2474),
// shared by a scene's own update graph (runtime.cu) and batched updates
// (batch.cu).
#pragma once

#include <cuda_runtime.h>

#include "apic_internal.h"

namespace apic {

// Substep size (src/apic.rs:2433-2441) and the loop condition (:2432).
__device__ __forceinline__ void plan(Ctl* ctl) {
    float t = ctl->t, frame = ctl->frame_dt;
    if (!(t < frame)) { ctl->go = 0; return; }
    float vmax = __uint_as_float(ctl->vmax_bits);
    float safe = vmax > 1e-5f ? ctl->cfl_cs / vmax : frame;
    float step = fminf(safe, frame - t);
    if (!(step > 0.0f) || ctl->substeps >= 100000u) {  // the reference would loop forever
        ctl->status |= kStatusBadStep;
        ctl->go = 0;
        return;
    }
    ctl->dt = step;
    ctl->go = 1;
    ctl->sort_now = (!(ctl->flags & APIC_UPDATE_DISABLE_SORT) && t == 0.0f) ? 1u : 0u;
    if (ctl->sort_now) ctl->sorted = 1;
    ctl->vmax_bits = 0;    // the coming G2P reduces the next maximum
    ctl->nonfinite = 0;
}

// End of a substep (src/apic.rs:2463-2467), then plan the next one.
__device__ __forceinline__ void advance(Ctl* ctl) {
    ctl->t = ctl->t + ctl->dt;
    ctl->prev_dt = ctl->dt;
    ctl->timestamp += 1;
    ctl->substeps += 1;
    plan(ctl);
}

}  // namespace apic
