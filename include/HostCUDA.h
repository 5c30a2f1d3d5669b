/*
 * Drop-in GPU boundary for ChaNGa's gravity force evaluation.
 *
 * Every entry point below replaces the function of the same name and
 * signature in the reference's HostCUDA.h (cited per declaration), so
 * TreePiece, ListCompute and DataManager call this library unchanged.  The
 * declarations are given C linkage (extern "C") so any FFI can bind them;
 * the library additionally exports the C++-mangled names the reference's
 * own header produces, so an unmodified ChaNGa object file links too.
 *
 * Semantics kept from the reference:
 *   - everything is asynchronous on the request's stream;
 *   - host arrays in a request (list, markers, starts, sizes, missed*) are
 *     owned by the caller and must stay valid until the completion callback;
 *     the library finishes reading them before it signals completion;
 *   - results ACCUMULATE into d_localVars (+= for a and potential, max for
 *     dtGrav); DataManagerTransferLocalTree zeroes them;
 *   - completion is signalled through the registered completion hook
 *     (changa_gb300_set_completion_hook, the stand-in for hapiAddCallback);
 *   - a CUDA error prints the failing call and aborts, unless the error mode
 *     is set to CHANGA_ERRORS_RECORD (changa_gb300.h).
 * What differs on purpose: per-request device temporaries come from the
 * stream-ordered allocator (cudaMallocAsync/cudaFreeAsync) instead of
 * cudaMalloc/cudaFree, so no entry point synchronises the device.
 */
#ifndef CHANGA_GB300_HOST_CUDA_H_
#define CHANGA_GB300_HOST_CUDA_H_

#include <stddef.h>
#include <cuda_runtime_api.h>
#include "cuda_typedef.h"

#ifndef __cplusplus
#include <stdbool.h>
#endif

/* Launch-shape constants of the reference (HostCUDA.h:8-22).  Kept for
 * source compatibility; the kernels here choose their own shapes. */
#define THREADS_PER_BLOCK 128
#define PARTS_PER_BLOCK 16
#define NODES_PER_BLOCK (THREADS_PER_BLOCK / PARTS_PER_BLOCK)
#define THREADS_PER_BLOCK_PART 128
#define PARTS_PER_BLOCK_PART 16
#define NODES_PER_BLOCK_PART (THREADS_PER_BLOCK_PART / PARTS_PER_BLOCK_PART)
#define NUM_INIT_MOMENT_INTERACTIONS_PER_BUCKET 100
#define NUM_INIT_PARTICLE_INTERACTIONS_PER_BUCKET 100

/** One gravity request (reference: HostCUDA.h:31-89, !GPU_LOCAL_TREE_WALK).
 *  list holds ILCell entries for both cell lists and flattened particle
 *  lists; bucketMarkers[numBucketsPlusOne] are CSR offsets into list;
 *  bucketStarts/bucketSizes give each bucket's targets in d_localParts. */
typedef struct _CudaRequest {
  cudaStream_t stream;
  CudaMultipoleMoments *d_localMoments;
  CudaMultipoleMoments *d_remoteMoments;
  CompactPartData *d_localParts;
  CompactPartData *d_remoteParts;
  VariablePartData *d_localVars;
  size_t sMoments;
  size_t sCompactParts;
  size_t sVarParts;
  void *list;
  int *bucketMarkers;
  int *bucketStarts;
  int *bucketSizes;
  int numInteractions;
  int numBucketsPlusOne;
  void *tp;
  void *missedNodes;
  void *missedParts;
  size_t sMissed;
  int *affectedBuckets;
  void *cb;
  void *state;
  cudatype fperiod;
  bool node;
  bool remote;
} CudaRequest;

/** Device pointers of one request (reference: HostCUDA.h:92-97). */
typedef struct _CudaDevPtr {
  void *d_list;
  int *d_bucketMarkers;
  int *d_bucketStarts;
  int *d_bucketSizes;
} CudaDevPtr;

/* CHANGA_GB300_NO_PROTOTYPES leaves out the C-linkage prototypes; the
 * library's C++-linkage forwarders (csrc/cxx_abi.cpp) define the reference's
 * mangled names and must not see them. */
#ifndef CHANGA_GB300_NO_PROTOTYPES
#ifdef __cplusplus
extern "C" {
#endif

/* reference: HostCUDA.h:99 / HostCUDA.cu:66-83.  size 0 sets *ptr = NULL. */
void allocatePinnedHostMemory(void **ptr, size_t size);
/* reference: HostCUDA.h:100 / HostCUDA.cu:85-101 */
void freePinnedHostMemory(void *ptr);

/* reference: HostCUDA.h:102-107 / HostCUDA.cu:115-149.  Allocates the three
 * persistent device arrays into *d_localMoments, *d_compactParts,
 * *d_varParts (freed by the caller with cudaFree), copies the host arrays,
 * zeroes the first numParticles result rows and signals callback. */
void DataManagerTransferLocalTree(void *moments, size_t sMoments,
                                  void *compactParts, size_t sCompactParts,
                                  void *varParts, size_t sVarParts,
                                  void **d_localMoments, void **d_compactParts,
                                  void **d_varParts, cudaStream_t stream,
                                  int numParticles, void *callback);

/* reference: HostCUDA.h:108-112 / HostCUDA.cu:158-183 */
void DataManagerTransferRemoteChunk(void *moments, size_t sMoments,
                                    void *compactParts, size_t sCompactParts,
                                    void **d_remoteMoments, void **d_remoteParts,
                                    cudaStream_t stream, void *callback);

/* reference: HostCUDA.h:114 / HostCUDA.cu:623-630 */
void TransferParticleVarsBack(VariablePartData *hostBuffer, size_t size,
                              void *d_varParts, cudaStream_t stream, void *cb);

/* Cell (quadrupole) lists against local, remote and missed moments.
 * reference: HostCUDA.h:116-118 / HostCUDA.cu:190-341 */
void TreePieceCellListDataTransferLocal(CudaRequest *data);
void TreePieceCellListDataTransferRemote(CudaRequest *data);
void TreePieceCellListDataTransferRemoteResume(CudaRequest *data);

/* Particle lists against local, caller-supplied, remote and missed
 * particles.  reference: HostCUDA.h:121-124 / HostCUDA.cu:345-572 */
void TreePiecePartListDataTransferLocal(CudaRequest *data);
void TreePiecePartListDataTransferLocalSmallPhase(CudaRequest *data,
                                                  CompactPartData *parts, int len);
void TreePiecePartListDataTransferRemote(CudaRequest *data);
void TreePiecePartListDataTransferRemoteResume(CudaRequest *data);

/* reference: CudaFunctions.h:7-8 / HostCUDA.cu:578-613: copy a request's
 * list, markers, starts and sizes to the device / release them (stream-
 * ordered; Cleanup takes the stream the Basic call used). */
void TreePieceDataTransferBasic(CudaRequest *data, CudaDevPtr *ptr);
void TreePieceDataTransferBasicCleanup(CudaDevPtr *ptr);

#ifdef __cplusplus
}
#endif
#endif /* CHANGA_GB300_NO_PROTOTYPES */

#endif /* CHANGA_GB300_HOST_CUDA_H_ */
