/*
 * Drop-in GPU boundary for ChaNGa's periodic Ewald correction.
 *
 * Replaces the reference's EwaldCUDA.h (declarations at EwaldCUDA.h:59-62,
 * implementation in HostCUDA.cu:1887-2192).  Struct layouts are identical
 * in both builds (HEXADECAPOLE defined or not, as the reference's own
 * header).  C linkage, with the reference's C++-mangled names exported as
 * well (see HostCUDA.h).
 *
 * Difference on purpose: the reference copies EwaldReadOnlyData and the
 * h-table into __constant__ symbols per call (HostCUDA.cu:1934-1935), which
 * races when two streams call EwaldHost concurrently.  Here both travel as
 * kernel parameters, so concurrent calls on different streams are safe.
 */
#ifndef CHANGA_GB300_EWALD_CUDA_H_
#define CHANGA_GB300_EWALD_CUDA_H_

#include "HostCUDA.h"

#define NEWH 80
#define BLOCK_SIZE 128

/** One Fourier-space term (reference: EwaldCUDA.h:11-14). */
typedef struct {
  cudatype hx, hy, hz;
  cudatype hCfac, hSfac;
} EwtData;

/** Root mass and centre, with the quadrupole moments in the quadrupole
 *  build (reference: EwaldCUDA.h:18-24). */
typedef struct {
#ifndef HEXADECAPOLE
  cudatype xx, xy, xz, yy, yz, zz;
#endif
  cudatype totalMass;
  cudatype cmx, cmy, cmz;
} MultipoleMomentsData;

/** Complete root moments, the hexadecapole build's Ewald expansion
 *  (reference: EwaldCUDA.h:28-36; unused by the quadrupole build). */
typedef struct {
  cudatype m;
  cudatype xx, yy, xy, xz, yz;
  cudatype xxx, xyy, xxy, yyy, xxz, yyz, xyz;
  cudatype xxxx, xyyy, xxxy, yyyy, xxxz, yyyz, xxyy, xxyz, xyyz;
  cudatype zz;
  cudatype xzz, yzz, zzz;
  cudatype xxzz, xyzz, xzzz, yyzz, yzzz, zzzz;
} MomcData;

/** Ewald parameters (reference: EwaldCUDA.h:40-47). */
typedef struct {
  MultipoleMomentsData mm;
  MomcData momcRoot;
  int n, nReps, nEwReps, nEwhLoop;
  cudatype L, fEwCut, alpha, alpha2, k1, ka, fEwCut2, fInner2;
} EwaldReadOnlyData;

/** Host buffers of one Ewald call (reference: EwaldCUDA.h:50-57). */
typedef struct {
  int EwaldRange[2];
  int *EwaldMarkers;
  EwtData *ewt;
  EwaldReadOnlyData *cachedData;
} EwaldData;

#ifndef CHANGA_GB300_NO_PROTOTYPES
#ifdef __cplusplus
extern "C" {
#endif

/* reference: EwaldCUDA.h:59 / HostCUDA.cu:1887-1894 (pinned buffers) */
void EwaldHostMemorySetup(EwaldData *h_idata, int size, int nEwhLoop, int largephase);
/* reference: EwaldCUDA.h:60 / HostCUDA.cu:1896-1901 */
void EwaldHostMemoryFree(EwaldData *h_idata, int largephase);
/* reference: EwaldCUDA.h:61-62 / HostCUDA.cu:1917-1956.  largephase != 0:
 * the particles EwaldMarkers[0..n) of d_localParts; otherwise the range
 * EwaldRange[0]..EwaldRange[1].  Accumulates into d_localVars. */
void EwaldHost(CompactPartData *d_localParts, VariablePartData *d_localVars,
               EwaldData *h_idata, cudaStream_t stream, void *cb, int myIndex,
               int largephase);

#ifdef __cplusplus
}
#endif
#endif /* CHANGA_GB300_NO_PROTOTYPES */

#endif /* CHANGA_GB300_EWALD_CUDA_H_ */
