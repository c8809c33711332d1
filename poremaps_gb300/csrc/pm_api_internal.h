// Host-side helpers shared by the C-ABI translation units.
#pragma once

#include <cuda_runtime.h>

#include "../../include/poremaps.h"

namespace pm {

pm_status set_error(pm_status st, const char* fmt, ...);
pm_status cuda_error(cudaError_t e, const char* where);
pm_status write_log_row(const char* path, bool first, int iteration, double conv, double tps,
                        const pm_result& r);
size_t problem_device_bytes(const pm_params* p);
const pm_params* problem_params(const pm_problem* pr);
long long problem_nvox(const pm_problem* pr);
cudaStream_t problem_stream(const pm_problem* pr);

}  // namespace pm
