// ln and cos for the Box-Muller transform of the hash RNG.
#pragma once
#include <math.h>

#ifndef SP_HD
#define SP_HD __host__ __device__ __forceinline__
#endif

namespace sp {

SP_HD double cr_log(double x, unsigned* hard) {
    (void)hard;
    return log(x);
}

SP_HD double cr_cos(double x, unsigned* hard) {
    (void)hard;
    return cos(x);
}

}  // namespace sp
