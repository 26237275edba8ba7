// host.h -- host-side helpers shared by the library's translation units.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "decaes_gpu.h"

namespace dh {

std::vector<double> julia_range(double start, double stop, int len);
std::vector<double> julia_logrange(double a, double b, int len);
double erfinv(double x);
std::string jlfmt(double v);
std::string check_t2map(const decaes_t2map_opts &o);
std::string check_t2part(const decaes_t2part_opts &o);

struct T2partPlan {
    std::vector<double> t2, logt2, weights;  // weights empty unless Sigmoid is given
    int sp0, sp1, mp0, mp1;                  // 0-based inclusive window index ranges
};
std::string t2part_plan(const decaes_t2part_opts &o, T2partPlan &p);

int mock_image(const decaes_mock_opts &o, uint64_t seed, void *image, int dtype, int nthreads);

// Raises a kernel's dynamic shared-memory limit to at least `bytes` on the
// current device, never lowering it; returns the cudaError_t value (defined
// in decaes_gpu.cu).
int raise_smem_limit(const void *kern, size_t bytes);

}  // namespace dh
