// Shared by the host translation units of libvoce_gpu.so; not part of the ABI.
#pragma once

namespace voce {

// Sets the message voce_last_error() returns; returns code.
int set_error(int code, const char *msg);

// Whether an RVE of this grid and precision is created without timing FFT
// tiles (the choice is cached for the shape, or tuning is off).
bool tiles_known(const int dims[3], int precision);

}  // namespace voce
