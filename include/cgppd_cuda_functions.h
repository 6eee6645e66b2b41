/*
 * cgppd_cuda_functions.h -- drop-in C ABI for the reference's CUDA energy module.
 *
 * Same names, arguments and meaning as the reference's src/cudaExterns.h:14-90 and
 * src/CudaFunctions.cu, so the reference's Replica / Simulation / tests link against
 * libcgppd_gb300.so unchanged.  Every entry point records failures (stderr + the
 * thread's last status, see cgppd_get_last_error) instead of exiting the process.
 */
#ifndef CGPPD_CUDA_FUNCTIONS_H_
#define CGPPD_CUDA_FUNCTIONS_H_

#include <cuda_runtime.h>

#ifdef __cplusplus
class AminoAcids; /* layout of src/AminoAcids.h:7-27; see cgppd_amino_acids.h */
extern "C" {
#else
typedef struct AminoAcids AminoAcids;
#endif

/* Replaces __throwLastCudaError (src/CudaFunctions.cu:20-32, declared
 * src/cudaExterns.h:18): prints the last CUDA error and throws `errorMessage`
 * (a const char*) to a C++ caller. */
void __throwLastCudaError(const char *errorMessage, const char *file, const int line);

/* Replaces LJPotentialDataToDevice (src/CudaFunctions.cu:75-104,
 * src/cudaExterns.h:20): device copy of a->LJpotentials[20][20] (raw RT values). */
float *LJPotentialDataToDevice(AminoAcids *a);

/* Replaces copyLJPotentialDataToDevice (src/CudaFunctions.cu:106-125,
 * src/cudaExterns.h:21): copy the table into a caller-allocated device buffer. */
void copyLJPotentialDataToDevice(float *dev_LJPotentialData, AminoAcids *a);

/* Replaces CUDA_EonDevice (src/CudaFunctions.cu:198-277, src/cudaExterns.h:29):
 * total non-bonded energy (kcal/mol) of the packed replica, written to *result (host).
 * pos/meta are device arrays of datasetSize float4 records.  LJPotentials is accepted
 * and never dereferenced; the table bound with bindLJTexture is used. */
void CUDA_EonDevice(float4 *residuePositions, float4 *residueMeta, int *residueCount, int *moleculePositions,
                    int *moleculeCount, float *LJPotentials, double *result, int blockSize, int datasetSize,
                    int sharedMemSize);

/* Replaces CUDA_EonDeviceNC (src/CudaFunctions.cu:724-754, src/cudaExterns.h:30):
 * as CUDA_EonDevice over non-crowder residues of different molecules only. */
void CUDA_EonDeviceNC(float4 *residuePositions, float4 *residueMeta, int *residueCount, int *moleculePositions,
                      int *moleculeCount, float *LJPotentials, double *result, int blockSize, int datasetSize,
                      int sharedMemSize);

/* Replaces CUDA_EonDevice_async (src/CudaFunctions.cu:176-190, src/cudaExterns.h:42):
 * enqueue the energy on `stream`; device_result (resultSize*resultSize floats) receives
 * the total in element 0 and zeros elsewhere, so the caller's host sum is unchanged.
 * Like the reference's asynchronous call it reports nothing back to the host: a residue
 * type outside 0..19 is read as type 0 without an error (the synchronous entry points
 * check the types and fail on such input).  On a stream other than the legacy default
 * one the launch is a programmatic dependent launch that waits for the stream's previous
 * kernel before touching memory (plain stream ordering). */
void CUDA_EonDevice_async(float4 *residuePositions, float4 *residueMeta, int *residueCount, int *moleculePositions,
                          int *moleculeCount, float *LJPotentials, float *device_result, int resultSize,
                          int blockSize, int datasetSize, int sharedMemSize, cudaStream_t stream);

/* Replaces CUDA_setBoxDimension / CUDA_freeBoxDimension (src/CudaFunctions.cu:157-167,
 * src/cudaExterns.h:45-46): periodic box edge for the current device (0 = open box). */
void CUDA_setBoxDimension(float value);
void CUDA_freeBoxDimension(void);

/* Replaces bindLJTexture / unbindLJTexture (src/CudaFunctions.cu:36-47,
 * src/cudaExterns.h:51-52): select the contact table the kernels read on the current
 * device. */
void bindLJTexture(float *ljp);
void unbindLJTexture(void);

/* No counterpart in the reference.  CUDA_EonDevice for callers that cannot allocate
 * device memory while they evaluate energies (code running inside another
 * framework's memory pool or under a fixed device-memory budget, or a loop that must
 * stay free of allocation calls): same arguments and result, but its scratch is a
 * static 139,896-byte device array owned by the library, so it calls no cudaMalloc or
 * cudaFree.  datasetSize is limited to 16384 residues (larger sizes are rejected with
 * an error and *result = 0).  Every call looks up the array's device address on the
 * current device (a lookup allocates nothing, and stays right after cudaDeviceReset);
 * the first call on a device may load the library's device code there and should come
 * before any stream capture.  All calls on a device share that device's array; calls
 * whose kernels overlapped on the GPU would race, so this function serialises its own
 * calls per device and returns after its kernel has finished. */
void CUDA_EonDevice_noalloc(float4 *residuePositions, float4 *residueMeta, int *residueCount,
                            int *moleculePositions, int *moleculeCount, float *LJPotentials, double *result,
                            int blockSize, int datasetSize, int sharedMemSize);

/* Library extension (no reference counterpart): {LJ raw, DH raw, total} of the last
 * synchronous call on the current device.  Returns 0 on success. */
int cgppd_last_energy_components(double *out3);

/* Run-time form of the reference's compile-time REPULSIVE_CROWDING switch
 * (src/definitions.h:18, off in its default build; src/CudaFunctions.cu:335-338 and
 * :492-498): when on, every pair with a crowder residue (meta.w == -1) contributes
 * (6/r)^12 in RT units below 15 A and no Debye-Hueckel term, in every later energy
 * call of the process (CUDA_EonDevice, _async, _noalloc).  Returns the previous
 * setting (0 off, 1 on). */
int cgppd_set_repulsive_crowding(int on);

/* Library extension: the calling thread's last error code (0 = none) and message;
 * clears it. */
int cgppd_get_last_error(char *buf, int buflen);

#ifdef __cplusplus
}
#endif

#endif /* CGPPD_CUDA_FUNCTIONS_H_ */
