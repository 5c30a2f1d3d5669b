/*
 * Byte layouts that cross the gravity GPU boundary.
 *
 * These are the structs ChaNGa's host code fills and hands to the GPU entry
 * points (cuda_typedef.h:55-272 in the reference, quadrupole build, no GPU
 * tree walk).  The layouts here are identical field for field so a ChaNGa
 * build compiled against this header passes the same bytes; the static
 * asserts in changa_gb300/csrc/abi_check.cu pin every size and offset.
 * They are plain C structs: the reference's C++ converting constructors are
 * host conveniences and do not change the layout.
 */
#ifndef CHANGA_GB300_CUDA_TYPEDEF_H_
#define CHANGA_GB300_CUDA_TYPEDEF_H_

/** Floating-point type on the GPU boundary (reference: cuda_typedef.h:12). */
typedef float cudatype;

/* Request-size thresholds in millions of interactions at which the host
 * flushes a request (reference: cuda_typedef.h:17-25). */
#define NODE_INTERACTIONS_PER_REQUEST_L 1.0
#define PART_INTERACTIONS_PER_REQUEST_L 0.1
#define NODE_INTERACTIONS_PER_REQUEST_RNR 1.0
#define PART_INTERACTIONS_PER_REQUEST_RNR 0.1
#define NODE_INTERACTIONS_PER_REQUEST_RR 1.0
#define PART_INTERACTIONS_PER_REQUEST_RR 0.1

#define TP_LARGE_PHASE_THRESHOLD_DEFAULT 0.0
#define AVG_SOURCE_PARTICLES_PER_ACTIVE 10

/** 3-vector (reference: cuda_typedef.h:55-77). */
typedef struct CudaVector3D {
  cudatype x, y, z;
} CudaVector3D;

/** Multipole moments of one tree node (reference: cuda_typedef.h:104-177,
 *  !GPU_LOCAL_TREE_WALK).
 *  Quadrupole build, 48 bytes: xx..zz are the raw second moments
 *  sum m dx dx about cm (not trace-free).
 *  HEXADECAPOLE build, 108 bytes: the scaled reduced (trace-free) moments
 *  up to fourth order of moments.h's FMOMR, in units of the node radius. */
typedef struct CudaMultipoleMoments {
  cudatype radius;
  cudatype soft;
  cudatype totalMass;
  CudaVector3D cm;
#ifdef HEXADECAPOLE
  cudatype xx, xy, xz, yy, yz;
  cudatype xxx, xyy, xxy, yyy, xxz, yyz, xyz;
  cudatype xxxx, xyyy, xxxy, yyyy, xxxz, yyyz, xxyy, xxyz, xyyz;
#else
  cudatype xx, xy, xz, yy, yz, zz;
#endif
} CudaMultipoleMoments;

/** A bucket of source particles on an interaction list
 *  (reference: cuda_typedef.h:208-221). */
typedef struct ILPart {
  int index;  /**< first particle of the bucket on the GPU */
  int off;    /**< replica code, bits 22-30 (see encodeOffset) */
  int num;    /**< particles in the bucket */
} ILPart;

/** A cell (or, for flattened particle lists, one source particle) on an
 *  interaction list (reference: cuda_typedef.h:225-235). */
typedef struct ILCell {
  int index;     /**< moment (or particle) index on the GPU */
  int offsetID;  /**< replica code in bits 22-30: x+3 | (y+3)<<3 | (z+3)<<6 */
} ILCell;

/** Particle data read by the force kernels, 20 bytes
 *  (reference: cuda_typedef.h:240-263). */
typedef struct CompactPartData {
  cudatype mass;
  cudatype soft;
  CudaVector3D position;
} CompactPartData;

/** Per-particle results, 20 bytes (reference: cuda_typedef.h:268-272).
 *  Kernels accumulate: a and potential with +=, dtGrav with max. */
typedef struct VariablePartData {
  CudaVector3D a;
  cudatype potential;
  cudatype dtGrav;
} VariablePartData;

#endif /* CHANGA_GB300_CUDA_TYPEDEF_H_ */
