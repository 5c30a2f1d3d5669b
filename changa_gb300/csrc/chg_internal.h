/*
 * Internal interfaces shared by the CUDA translation units of the gravity
 * library (not part of the public C-ABI in include/).
 */
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "cuda_typedef.h"
#include "changa_gb300.h"

namespace chg {

enum Form : int { kF32 = 0, kF64 = 1, kMix = 2 };

/* Arguments of one interaction-list launch. */
struct ListArgs {
  const void* src;      // kF32: CudaMultipoleMoments* or CompactPartData*
                        // kF64: double* (12 or 5 per row); kMix: packed float4
  long long n_src;
  const void* tgt;      // kF32: CompactPartData*; kF64: double*; kMix: packed float4
  long long n_tgt;
  void* vars;           // kF32: VariablePartData*; kF64/kMix: double* (5 per row)
  const int2* list;     // ILCell {index, offsetID}
  long long n_entries;  // entries in list (markers are clamped to it)
  const int* markers;   // n_buckets + 1
  const int* starts;
  const int* sizes;
  int n_buckets;
  float fperiod_f;
  double fperiod_d;
  unsigned int* queue;  // work counter, zero at launch
};

/* Packed FP32-mixed layouts (built by pack kernels from FP64 inputs):
 *   cell   : 4 float4 per node  {hi.xyz, M} {lo.xyz, soft} {xx,xy,xz,yy}
 *            {yz, zz, tr, 0}
 *   particle: 2 float4 per particle {hi.xyz, mass} {lo.xyz, soft}
 * hi = (float)x, lo = (float)(x - hi), both exact in FP64. */
constexpr int kCellPackF4 = 4;
constexpr int kPartPackF4 = 2;
/* hexadecapole cell: {hi.xyz, M} {lo.xyz, soft} then the radius and the 21
 * scaled reduced moments (xx xy xz yy yz, xxx xyy xxy yyy xxz yyz xyz,
 * xxxx xyyy xxxy yyyy xxxz yyyz xxyy xxyz xyyz) and two zeros */
constexpr int kCellHexPackF4 = 8;

/* launchers (grav_lists.cu) */
cudaError_t launch_list(int form, bool cell, const ListArgs& a, cudaStream_t s);
int list_variant_count();
int set_list_variant(int kernel, int variant);
int get_list_variant(int kernel);
int set_hex_variant(int v);
int get_hex_variant();
/* poll limit of the TMA variants' mbarrier waits (negative: the default) */
void set_tma_wait_polls(int polls);
/* TMA-variant launches since load */
unsigned long long tma_launches();
/* Synchronises the current device, then returns (in bits) and clears the
 * library's device status word (bit 0: a TMA wait ran out). */
cudaError_t read_device_status(unsigned* bits);
cudaError_t launch_pack_cells(const double* moments, long long n, float4* out, cudaStream_t s);
cudaError_t launch_pack_parts(const double* parts, long long n, float4* out, cudaStream_t s);
cudaError_t launch_zero_vars_f32(VariablePartData* v, long long n, cudaStream_t s);
/* hexadecapole build: cell lists over 27-double (kF64) or packed (kMix)
 * moments; the pack; cells as point-mass particles {M, soft, cm} */
cudaError_t launch_list_hex(int form, const ListArgs& a, cudaStream_t s);
cudaError_t launch_pack_cells_hex(const double* moments, long long n, float4* out, cudaStream_t s);
cudaError_t launch_cells_as_parts(const double* moments, int stride, long long n, double* out,
                                  cudaStream_t s);

/* Ewald (ewald.cu) */
struct EwaldArgsF32;  // defined in ewald.cu
cudaError_t launch_ewald_f32(const CompactPartData* parts, VariablePartData* vars,
                             const int* markers, int largephase, int first, int last,
                             const EwaldReadOnlyData& ro, const EwtData* ewt,
                             cudaStream_t s);
/* hex: the hexadecapole build's expansion (p.momc required) */
cudaError_t launch_ewald_fp(int form, const double* parts, long long n_parts, const int* idx,
                            long long n_idx, const ChangaEwaldParams& p, double* vars,
                            cudaStream_t s, bool hex = false);

/* adjoint of the Ewald term (quadrupole root expansion, FP64): adds the
 * vector-Jacobian product of lam . a_ewald to grad (n x 4 {dL/dx, dL/dm});
 * acc: 10 doubles of device scratch */
cudaError_t launch_ewald_vjp(const double* parts, long long n_parts, const ChangaEwaldParams& p,
                             const double* lam, double* grad, double* acc, cudaStream_t s);

/* runtime helpers (hostcuda.cu) */
int sm_count();
void count_launch(unsigned n = 1);
/* Keeps memory freed with cudaFreeAsync cached in this device's default
 * pool (a process-local pool attribute, set once per device). */
void prepare_pool();
int record_error(int code, const char* what, const char* file, int line);

/* Kernel ids for the optional per-kernel event timing
 * (changa_gb300_set_timing / changa_gb300_kernel_time). */
enum KernelId : int {
  kKidListF32Cell = 0, kKidListF32Part, kKidListF64Cell, kKidListF64Part, kKidListMixCell,
  kKidListMixPart, kKidEwaldF32, kKidEwaldF64, kKidEwaldMix, kKidPack, kKidVjpCell, kKidVjpPart,
  kKidMoments, kKidCount
};
inline int list_kernel_id(int form, bool cell) { return 2 * form + (cell ? 0 : 1); }

/* Records CUDA events around one launch on stream s when timing is on. */
struct TimingScope {
  TimingScope(int kid, cudaStream_t s);
  ~TimingScope();
  int kid;
  cudaStream_t s;
  void* start;
};

}  // namespace chg

#define CHG_CUDA(call)                                                            \
  do {                                                                            \
    cudaError_t e_ = (call);                                                      \
    if (e_ != cudaSuccess) return ::chg::record_error((int)e_, #call, __FILE__, __LINE__); \
  } while (0)
