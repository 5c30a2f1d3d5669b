/*
 * CPU oracle API for the gravity hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Two libraries implement this header:
 *   - oracle/_ref/libchanga_ref.so : ChaNGa's own gravity.h (SPLINEQ,
 *     SPLINE, nodeBucketForce, partBucketForce) and Ewald.cpp (EwaldInit,
 *     BucketEwald) compiled unchanged against oracle/shim (ref_driver.cpp).
 *     Built only where the reference sources are present.
 *   - oracle/_build/libchanga_port.so : grav_oracle.c, this project's plain
 *     C restatement of the same functions, pinned against the former and
 *     against tests/golden.  It is the oracle wherever the reference sources
 *     are absent, and the timed CPU baseline.
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * either library; the product never does.
 *
 * Layouts (all FP64 mirrors of the boundary structs in include/cuda_typedef.h):
 *   moments  : 12 doubles per node  {radius, soft, totalMass, cm.x, cm.y,
 *              cm.z, xx, xy, xz, yy, yz, zz}   (CudaMultipoleMoments order)
 *   parts    : 5 doubles per particle {mass, soft, x, y, z} (CompactPartData)
 *   vars     : 5 doubles per particle {a.x, a.y, a.z, potential, dtGrav}
 *              (VariablePartData); results ACCUMULATE (+= and max) as the
 *              reference does (gravity.h:293-298, 460-472, Ewald.cpp:275-279).
 *   list     : int32 pairs {index, offsetID} (ILCell); the periodic replica
 *              is bits 22-30 of offsetID (TreePiece.cpp:3631-3652).
 *   markers  : CSR offsets into list per bucket, starts/sizes: target range
 *              of each bucket in the particle array.
 */
#ifndef CHANGA_ORACLE_API_H
#define CHANGA_ORACLE_API_H

#ifdef __cplusplus
extern "C" {
#endif

/* Potential energy 0.5 sum_i m_i phi_i of an open system by FP64 direct
 * summation with partBucketForce's spline softening (port only). */
double oracle_direct_energy(const double* parts, long n, int nthreads);

/* Cell (quadrupole multipole) interaction lists: nodeBucketForce per entry.
 * bucket_ids (may be NULL) restricts the work to those buckets. */
int oracle_cell_list_forces(const double* moments, long n_moments,
                            const double* parts, long n_parts,
                            const int* list, const int* markers,
                            const int* starts, const int* sizes, int n_buckets,
                            const int* bucket_ids, int n_ids,
                            double fperiod, double* vars, int nthreads);

/* Particle interaction lists (flattened to one entry per source particle):
 * partBucketForce per entry. */
int oracle_part_list_forces(const double* sources, long n_sources,
                            const double* targets, long n_targets,
                            const int* list, const int* markers,
                            const int* starts, const int* sizes, int n_buckets,
                            const int* bucket_ids, int n_ids,
                            double fperiod, double* vars, int nthreads);

/* Ewald h-loop table (EwaldInit): writes up to max_h rows of 5 doubles
 * {hx, hy, hz, hCfac, hSfac}; returns nEwhLoop or -1 if max_h too small. */
int oracle_ewald_table(const double* root_moments, double L, double dEwhCut,
                       double* ewt, int max_h);

/* Ewald correction (BucketEwald) for parts[idx[k]] into vars[k]
 * (idx may be NULL: k indexes parts directly, n_idx = count). */
int oracle_ewald_forces(const double* parts, long n_parts, const int* idx, long n_idx,
                        const double* root_moments, double L, int nReps,
                        double fEwCut, double dEwhCut, double* vars, int nthreads);

/* Hexadecapole build of the cell lists (nodeBucketForce with
 * HEXADECAPOLE): moments 27 per node {radius, soft, totalMass, cm.xyz, xx xy
 * xz yy yz, xxx xyy xxy yyy xxz yyz xyz, xxxx xyyy xxxy yyyy xxxz yyyz xxyy
 * xxyz xyyz} (scaled reduced moments); geom 10 per request bucket {cm.xyz,
 * soft, bbox lesser xyz, greater xyz} for the softening test.  Cells whose
 * softening meets the bucket act as softened point masses. */
int oracle_cell_list_forces_hex(const double* moments, long n_moments, const double* parts,
                                long n_parts, const int* list, const int* markers,
                                const int* starts, const int* sizes, int n_buckets,
                                const double* geom, double fperiod, double* vars, int nthreads);

/* Hexadecapole build of the Ewald correction: root_moments holds the 27
 * hexadecapole values of the root (layout as above).  The table function
 * also returns the root's complete moments (MomcData order, 32 doubles) in
 * momc when it is not NULL. */
int oracle_ewald_table_hex(const double* root_moments, double L, double dEwhCut, double* ewt,
                           int max_h, double* momc);
int oracle_ewald_forces_hex(const double* parts, long n_parts, const int* idx, long n_idx,
                            const double* root_moments, double L, int nReps, double fEwCut,
                            double dEwhCut, double* vars, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
