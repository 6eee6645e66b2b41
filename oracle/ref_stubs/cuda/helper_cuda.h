/* The two CUDA-samples error macros the reference's CUDA build uses (src/Replica.cpp,
 * src/Simulation.cpp), for linking the reference's own call sites against the drop-in
 * library.  TEST INFRASTRUCTURE ONLY.  getLastCudaError reports through the library's
 * __throwLastCudaError (src/cudaExterns.h), which throws on a pending CUDA error. */
#pragma once

#include <cuda_runtime.h>

extern "C" void __throwLastCudaError(const char *errorMessage, const char *file, const int line);

#define getLastCudaError(msg) __throwLastCudaError(msg, __FILE__, __LINE__)
#define checkCudaErrors(call) (call)
