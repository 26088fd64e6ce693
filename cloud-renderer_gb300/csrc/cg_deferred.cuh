// cg_deferred.cuh -- device-side declarations shared by the deferred renderer.
#pragma once

#include "cg_internal.h"
#include "cg_sample.cuh"

// Sun-cone schedule of a launch (k_trace.cu).
ConeSchedule make_cone_schedule(const VolDesc& vd, const TraceParams& tp);
