/*
 * The reference declares its GPU boundary with C++ linkage (HostCUDA.h:99-126,
 * EwaldCUDA.h:59-62; no extern "C"), so an unmodified ChaNGa object file
 * refers to the mangled names.  These forwarders define exactly those
 * names, with the reference's parameter types, so such objects link against
 * this library as well as code compiled against include/HostCUDA.h (which
 * binds the C names).  Both routes end in the same implementation.
 */
#define CHANGA_GB300_NO_PROTOTYPES
#include "HostCUDA.h"
#include "EwaldCUDA.h"

extern "C" {
void chg_impl_allocatePinnedHostMemory(void**, size_t);
void chg_impl_freePinnedHostMemory(void*);
void chg_impl_DataManagerTransferLocalTree(void*, size_t, void*, size_t, void*, size_t, void**,
                                           void**, void**, cudaStream_t, int, void*);
void chg_impl_DataManagerTransferRemoteChunk(void*, size_t, void*, size_t, void**, void**,
                                             cudaStream_t, void*);
void chg_impl_TransferParticleVarsBack(VariablePartData*, size_t, void*, cudaStream_t, void*);
void chg_impl_TreePieceCellListDataTransferLocal(CudaRequest*);
void chg_impl_TreePieceCellListDataTransferRemote(CudaRequest*);
void chg_impl_TreePieceCellListDataTransferRemoteResume(CudaRequest*);
void chg_impl_TreePiecePartListDataTransferLocal(CudaRequest*);
void chg_impl_TreePiecePartListDataTransferLocalSmallPhase(CudaRequest*, CompactPartData*, int);
void chg_impl_TreePiecePartListDataTransferRemote(CudaRequest*);
void chg_impl_TreePiecePartListDataTransferRemoteResume(CudaRequest*);
void chg_impl_TreePieceDataTransferBasic(CudaRequest*, CudaDevPtr*);
void chg_impl_TreePieceDataTransferBasicCleanup(CudaDevPtr*);
void chg_impl_EwaldHostMemorySetup(EwaldData*, int, int, int);
void chg_impl_EwaldHostMemoryFree(EwaldData*, int);
void chg_impl_EwaldHost(CompactPartData*, VariablePartData*, EwaldData*, cudaStream_t, void*, int,
                        int);
}

void allocatePinnedHostMemory(void** p, size_t s) { chg_impl_allocatePinnedHostMemory(p, s); }
void freePinnedHostMemory(void* p) { chg_impl_freePinnedHostMemory(p); }
void DataManagerTransferLocalTree(void* moments, size_t sMoments, void* compactParts,
                                  size_t sCompactParts, void* varParts, size_t sVarParts,
                                  void** d_localMoments, void** d_compactParts, void** d_varParts,
                                  cudaStream_t stream, int numParticles, void* callback) {
  chg_impl_DataManagerTransferLocalTree(moments, sMoments, compactParts, sCompactParts, varParts,
                                        sVarParts, d_localMoments, d_compactParts, d_varParts,
                                        stream, numParticles, callback);
}
void DataManagerTransferRemoteChunk(void* moments, size_t sMoments, void* compactParts,
                                    size_t sCompactParts, void** d_remoteMoments,
                                    void** d_remoteParts, cudaStream_t stream, void* callback) {
  chg_impl_DataManagerTransferRemoteChunk(moments, sMoments, compactParts, sCompactParts,
                                          d_remoteMoments, d_remoteParts, stream, callback);
}
void TransferParticleVarsBack(VariablePartData* hostBuffer, size_t size, void* d_varParts,
                              cudaStream_t stream, void* cb) {
  chg_impl_TransferParticleVarsBack(hostBuffer, size, d_varParts, stream, cb);
}
void TreePieceCellListDataTransferLocal(CudaRequest* d) { chg_impl_TreePieceCellListDataTransferLocal(d); }
void TreePieceCellListDataTransferRemote(CudaRequest* d) { chg_impl_TreePieceCellListDataTransferRemote(d); }
void TreePieceCellListDataTransferRemoteResume(CudaRequest* d) {
  chg_impl_TreePieceCellListDataTransferRemoteResume(d);
}
void TreePiecePartListDataTransferLocal(CudaRequest* d) { chg_impl_TreePiecePartListDataTransferLocal(d); }
void TreePiecePartListDataTransferLocalSmallPhase(CudaRequest* d, CompactPartData* p, int len) {
  chg_impl_TreePiecePartListDataTransferLocalSmallPhase(d, p, len);
}
void TreePiecePartListDataTransferRemote(CudaRequest* d) { chg_impl_TreePiecePartListDataTransferRemote(d); }
void TreePiecePartListDataTransferRemoteResume(CudaRequest* d) {
  chg_impl_TreePiecePartListDataTransferRemoteResume(d);
}
void TreePieceDataTransferBasic(CudaRequest* d, CudaDevPtr* p) { chg_impl_TreePieceDataTransferBasic(d, p); }
void TreePieceDataTransferBasicCleanup(CudaDevPtr* p) { chg_impl_TreePieceDataTransferBasicCleanup(p); }
void EwaldHostMemorySetup(EwaldData* h, int size, int nEwhLoop, int largephase) {
  chg_impl_EwaldHostMemorySetup(h, size, nEwhLoop, largephase);
}
void EwaldHostMemoryFree(EwaldData* h, int largephase) { chg_impl_EwaldHostMemoryFree(h, largephase); }
void EwaldHost(CompactPartData* d_localParts, VariablePartData* d_localVars, EwaldData* h,
               cudaStream_t stream, void* cb, int myIndex, int largephase) {
  chg_impl_EwaldHost(d_localParts, d_localVars, h, stream, cb, myIndex, largephase);
}
