// status.h -- error reporting shared by every entry point of the library.
//
// The reference's entry points call getLastCudaError, which prints and exits the
// process.  Here every failure is printed to stderr and recorded as the calling
// thread's last status; cgppd_get_last_error() returns and clears it, so a host
// (C++, ctypes, JNI) can turn it into its own exception.
#pragma once

#include <cuda_runtime.h>

#ifdef __cplusplus
extern "C" {
#endif

// Last recorded error of the calling thread: returns its code (0 = none), copies the
// message into buf (if non-null) and clears it.
int cgppd_get_last_error(char *buf, int buflen);

#ifdef __cplusplus
}
#endif

// Record `err` (if not cudaSuccess) with `where`; returns 0 on success, -1 otherwise.
int cgppd_check(cudaError_t err, const char *where);
// Record a library-level failure with message `msg`; returns -1.
int cgppd_fail(const char *msg);
