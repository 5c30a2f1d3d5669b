/*
 * Minimal stand-ins for the types that ChaNGa's gravity.h and Ewald.cpp
 * reference, so those two files compile unchanged as a CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY: this header is used by oracle/ref_driver.cpp,
 * which is built into oracle/_ref/ and is loaded only by tests and by the
 * CPU-baseline leg of bench.py.  Nothing in the product links it.
 *
 * The real headers these replace need Charm++ and the N-BodyShop utility
 * library (Vector3D.h, OrientedBox.h, Sphere.h, Space.h, SFC.h), neither of
 * which exists here.  Their include guards are pre-defined below so that the
 * reference's own GenericTreeNode.h, TreeNode.h and ParallelGravity.h become
 * empty when gravity.h / Ewald.cpp pull them in.  Only the members those two
 * files touch are provided.
 */
#ifndef CHANGA_ORACLE_REF_SHIM_H
#define CHANGA_ORACLE_REF_SHIM_H

#include <cmath>
#include <cassert>
#include <cstdlib>
#include <cstring>

/* Guards of the reference headers replaced here (GenericTreeNode.h:7,
 * TreeNode.h:7, ParallelGravity.h:4, MultipoleMoments.h:9). */
#define GENERICTREENODE_H
#define TREENODE_H
#define PARALLELGRAVITY_H
#define MULTIPOLEMOMENTS_H

#include "cosmoType.h"   /* the reference's own: cosmoType = double */

#define CkAssert(x) assert(x)

template <typename T>
struct Vector3D {
  T x, y, z;
  Vector3D() : x(0), y(0), z(0) {}
  Vector3D(T v) : x(v), y(v), z(v) {}
  Vector3D(T a, T b, T c) : x(a), y(b), z(c) {}
  template <typename U>
  Vector3D(const Vector3D<U>& o) : x(o.x), y(o.y), z(o.z) {}
  T lengthSquared() const { return x * x + y * y + z * z; }
  T length() const { return std::sqrt(lengthSquared()); }
  Vector3D& operator+=(const Vector3D& o) { x += o.x; y += o.y; z += o.z; return *this; }
  Vector3D& operator-=(const Vector3D& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
  Vector3D& operator=(T v) { x = y = z = v; return *this; }
  T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <typename T> inline Vector3D<T> operator+(const Vector3D<T>& a, const Vector3D<T>& b) { return Vector3D<T>(a.x + b.x, a.y + b.y, a.z + b.z); }
template <typename T> inline Vector3D<T> operator-(const Vector3D<T>& a, const Vector3D<T>& b) { return Vector3D<T>(a.x - b.x, a.y - b.y, a.z - b.z); }
template <typename T> inline Vector3D<T> operator-(const Vector3D<T>& a) { return Vector3D<T>(-a.x, -a.y, -a.z); }
template <typename T> inline Vector3D<T> operator*(const Vector3D<T>& a, T s) { return Vector3D<T>(a.x * s, a.y * s, a.z * s); }
template <typename T> inline Vector3D<T> operator*(T s, const Vector3D<T>& a) { return Vector3D<T>(a.x * s, a.y * s, a.z * s); }
template <typename T> inline Vector3D<T> operator/(const Vector3D<T>& a, T s) { return Vector3D<T>(a.x / s, a.y / s, a.z / s); }

template <typename T>
struct OrientedBox {
  Vector3D<T> lesser_corner, greater_corner;
};

template <typename T>
struct Sphere {
  Vector3D<T> origin;
  T radius;
  Sphere() : radius(0) {}
  Sphere(const Vector3D<T>& o, T r) : origin(o), radius(r) {}
};

#ifdef HEXADECAPOLE
#include "moments.h"  /* the reference's own FMOMR and momEvalFmomrcm */
/* Hexadecapole MultipoleMoments: the members gravity.h reads
 * (MultipoleMoments.h:182-185 layout with HEXADECAPOLE). */
struct MultipoleMoments {
  cosmoType radius;
  cosmoType soft;
  cosmoType totalMass;
  Vector3D<cosmoType> cm;
  FMOMR mom;
  MultipoleMoments() : radius(0), soft(0), totalMass(0) { std::memset(&mom, 0, sizeof(mom)); }
  cosmoType getRadius() const { return radius; }
};
#else
/* Quadrupole MultipoleMoments: the members gravity.h and Ewald.cpp read
 * (MultipoleMoments.h:182-187 layout, non-HEXADECAPOLE). */
struct MultipoleMoments {
  cosmoType radius;
  cosmoType soft;
  cosmoType totalMass;
  Vector3D<cosmoType> cm;
  double xx, xy, xz, yy, yz, zz;
  MultipoleMoments() : radius(0), soft(0), totalMass(0), xx(0), xy(0), xz(0), yy(0), yz(0), zz(0) {}
  cosmoType getRadius() const { return radius; }
};
#endif

class ExternalGravityParticle {
 public:
  cosmoType mass;
  cosmoType soft;
  Vector3D<cosmoType> position;
};

class GravityParticle : public ExternalGravityParticle {
 public:
  Vector3D<cosmoType> treeAcceleration;
  cosmoType potential;
  cosmoType dtGrav;
  cosmoType interMass;
  int rung;
  GravityParticle() : potential(0), dtGrav(0), interMass(0), rung(0) {}
};

namespace Tree {
enum NodeType {
  Invalid = 1, Bucket, Internal, Boundary, NonLocal, Empty, Top,
  NonLocalBucket, Cached, CachedBucket, CachedEmpty
};
class GenericTreeNode {
 public:
  NodeType myType;
  int firstParticle, lastParticle, particleCount;
  MultipoleMoments moments;
  OrientedBox<double> boundingBox;
  GenericTreeNode() : myType(Bucket), firstParticle(0), lastParticle(-1), particleCount(0) {}
  NodeType getType() const { return myType; }
};
}  // namespace Tree
using Tree::GenericTreeNode;

namespace TreeStuff {
/* TreeNode.h:35 */
const double opening_geometry_factor = 2 / sqrt(3.0);
}

/* EWT as in ParallelGravity.h:635-639. */
typedef struct ewaldTable {
  double hx, hy, hz;
  double hCfac, hSfac;
} EWT;

/* Charm++ message/proxy plumbing that EwaldInit() touches on its last
 * lines; the message is simply discarded. */
#define CK_QUEUEING_IFIFO 0
struct EwaldMsg {
  bool fromInit;
  static void* operator new(size_t sz, int) { return ::operator new(sz); }
  static void operator delete(void* p) { ::operator delete(p); }
  static void operator delete(void* p, int) { ::operator delete(p); }
};
static int g_shim_priority_slot[2];
inline void* CkPriorityPtr(EwaldMsg*) { return g_shim_priority_slot; }
inline void CkSetQueueing(EwaldMsg*, int) {}
struct ShimTreePieceElement {
  void calculateEwald(EwaldMsg* m) { delete m; }
};
struct ShimTreePieceProxy {
  ShimTreePieceElement e;
  ShimTreePieceElement& operator[](int) { return e; }
};

/* The TreePiece members BucketEwald()/EwaldInit() use
 * (ParallelGravity.h:1099, 1222-1231, 1599). */
class TreePiece {
 public:
  GravityParticle* myParticles;
  GenericTreeNode* root;
  Vector3D<cosmoType> fPeriod;
  int nReplicas;
  double fEwCut;
  double dEwhCut;
  EWT* ewt;
  int nMaxEwhLoop;
  int nEwhLoop;
  int activeRung;
  bool bBucketsInited;
  int thisIndex, numTreePieces, numChunks;
  ShimTreePieceProxy thisProxy;
#ifdef HEXADECAPOLE
  MOMC momcRoot; /* ParallelGravity.h: the root's complete moments */
#endif
  TreePiece()
      : myParticles(0), root(0), nReplicas(0), fEwCut(0), dEwhCut(0), ewt(0),
        nMaxEwhLoop(100), nEwhLoop(0), activeRung(0), bBucketsInited(true),
        thisIndex(0), numTreePieces(1), numChunks(1) {
    ewt = new EWT[nMaxEwhLoop];
  }
  ~TreePiece() { delete[] ewt; }
  void BucketEwald(GenericTreeNode* req, int nReps, double fEwCut);
  void EwaldInit();
  void EwaldGPU();
  void EwaldGPUComplete();
};

#endif
