// Host build of the device helper f32_of_difference, for the exactness test
// (tests/test_f32_diff.py compiles this with g++ and calls it through ctypes).
#include <cstddef>

#include "../cuspatial_gb300/csrc/f32_diff.cuh"

extern "C" void f32_of_differences(const double* x, const double* a, size_t n, float* out,
                                   int* ok)
{
  for (size_t i = 0; i < n; ++i) ok[i] = cspt::f32_of_difference(x[i], a[i], out[i]) ? 1 : 0;
}
