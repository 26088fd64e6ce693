// cg_deferred.cuh -- device-side declarations shared by the deferred renderer.
#pragma once

#include "cg_internal.h"
#include "cg_sample.cuh"

