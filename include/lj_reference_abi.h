/*
 * lj_reference_abi.h -- the reference's own CUDA entry points, reimplemented.
 *
 * vlvovch/lennard-jones-cuda splits its library between MDSystem.cpp (host)
 * and MDSystem.cu (device) through this extern "C" block, declared at
 * src/library/MDSystem.cpp:10-25 and defined at src/library/MDSystem.cu:155-299.
 * liblj_gb300.so exports the same symbols with the same signatures and
 * argument meanings, so the reference's MDSystem.cpp compiled with
 * USE_CUDA_TOOLKIT links against this library instead of its MDSystem.cu:
 * the force call then runs the sm_103a all-pairs kernel of this library
 * (fixed-point minimum image, FP32 pair math, compensated per-particle sums).
 *
 * Behavioural differences, by design:
 *  - no call exits the process: a CUDA failure is recorded and reported by
 *    lj_reference_abi_status() / lj_reference_abi_error() (the reference's
 *    checkCudaErrors prints and calls exit());
 *  - threadExit() synchronises and releases this layer's buffers; it does not
 *    reset the device for the whole process (MDSystem.cu:294-297);
 *  - `blockSize` (CUDABlockSize) selects the nearest i-block size of the
 *    kernel shapes; `q` stays unused as in the reference;
 *  - no per-call cudaMalloc/cudaFree: work buffers are cached per particle
 *    count (MDSystem.cu:265-287 allocated two RDF arrays on every call).
 */
#ifndef LJ_REFERENCE_ABI_H
#define LJ_REFERENCE_ABI_H

#ifdef __cplusplus
extern "C" {
#endif

/* MDSystem.cu:158-165: two device float4 arrays of numBodies each. */
void allocateNBodyArrays(float* vel[2], int numBodies);

/* MDSystem.cu:167-173: one device float4 array (4 floats per element). */
void allocateArray(float** dest, int number);

/* MDSystem.cu:175-179 */
void deleteNBodyArrays(float* vel[2]);

/* MDSystem.cu:181-184 */
void deleteArray(float* arr);

/* MDSystem.cu:186-192: device int array of `number` elements. */
void allocateIntArray(int** dest, int number);

/* MDSystem.cu:194-197 */
void deleteIntArray(int* arr);

/* MDSystem.cu:199-210: device float4[numBodies] -> host (pbo ignored). */
void copyArrayFromDevice(float* host, const float* device, unsigned int pbo, int numBodies);

/* MDSystem.cu:212-216: host float4[numBodies] -> device. */
void copyArrayToDevice(float* device, const float* host, int numBodies);

/* MDSystem.cu:218-226: OpenGL buffer registration, no-ops as in the reference. */
void registerGLBufferObject(unsigned int pbo);
void unregisterGLBufferObject(unsigned int pbo);

/* MDSystem.cu:228: device synchronisation. */
void threadSync(void);

/* MDSystem.cu:230-291.  Pos: device float4[numBodies] (w ignored); Force:
 * device float4[numBodies] out, xyz = LJ force (eps = sigma = 1), w =
 * sum_j (r^-12 - r^-6); *host_pressure = (2/3) sum over ordered pairs of
 * r^2 * (12 r^-14 - 6 r^-8) (the virial term before CalculateParameters adds
 * N T and divides by the volume); host_RDF (may be NULL): 256 ordered-pair
 * counts of floor(r^2 / host_dr2) with the overflow in bin 255.  Minimum
 * image applies when Lperiodic != 0. */
void calculateNForces(float* Pos, float* Force, float* host_pressure, int numBodies, float host_L,
                      int Lperiodic, int* host_RDF, float host_dr2, int blockSize, int q);

/* MDSystem.cu:294-297 (see above: no process-wide device reset). */
void threadExit(void);

/* Status of the last call of this layer: 0 = success, otherwise an lj_status
 * code (lj_gb300.h); the message of the last failure. */
int lj_reference_abi_status(void);
const char* lj_reference_abi_error(void);

#ifdef __cplusplus
}
#endif

#endif /* LJ_REFERENCE_ABI_H */
