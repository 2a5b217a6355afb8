// Shared by the host translation units of libvoce_gpu.so; not part of the ABI.
#pragma once

namespace voce {

// Sets the message voce_last_error() returns; returns code.
int set_error(int code, const char *msg);

}  // namespace voce
