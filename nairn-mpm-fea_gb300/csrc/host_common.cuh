// host_common.cuh -- host helpers shared by the single-run context
// (mpm_gpu.cu) and the batch/server translation unit (batch.cu).
#pragma once

#include <string>

#include "mpm_device.cuh"
#include "nairn_mpm_gpu.h"

namespace nmg {

constexpr int kParticleDoubles = 41;  // double columns of DevParticles besides zeta

// device material record of one MpmGpuMaterial (specific constants as the
// reference derives them); MPMGPU_OK or an error code with `why` set
int derive_material(const MpmGpuMaterial &in, int np, DevMat &m, std::string &why, int kterms);

// the host columns of MpmGpuParticles in device column order (nullptr for the
// natural coordinates)
void hcols(const MpmGpuParticles *h, double *out[kParticleDoubles]);

// sets the message of mpmgpu_last_error(NULL) and returns code
int fail_static(int code, const std::string &m);

}  // namespace nmg
