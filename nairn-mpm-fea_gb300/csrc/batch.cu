// batch.cu -- the batch (mpmgpu_batch_*) and serving (mpmgpu_server_*)
// entry points of include/nairn_mpm_gpu.h, compiled apart from the
// single-run context so the two kernel instantiation sets build in parallel.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "host_common.cuh"
#include "mpm_kernels.cuh"
#include "nairn_mpm_gpu.h"
#include "sort.cuh"

using namespace nmg;

namespace {
std::string g_static_err;  // the last creation error of a batch or server
}  // namespace

#include "batch.cuh"
#include "server.cuh"
