/*
 * Geometry predicates that ChaNGa's gravity.h calls through Space::
 * (gravity.h:256-259, 620-635, 676-722).  The original lives in the
 * N-BodyShop utility library, which is not available; these are this
 * project's own statements of the same predicates, with closed-ball
 * semantics (a touching sphere counts as intersecting).  The host walk in
 * changa_gb300/host/tree.cpp uses the identical predicates.
 *
 * TEST INFRASTRUCTURE ONLY (oracle/_ref build).
 */
#ifndef CHANGA_ORACLE_SPACE_H
#define CHANGA_ORACLE_SPACE_H

namespace Space {

/* Squared distance from the sphere centre to the nearest point of the box. */
template <typename T, typename T2>
inline double box_dist2(const OrientedBox<T>& b, const Sphere<T2>& s) {
  double d2 = 0.0, d;
  if ((d = b.lesser_corner.x - s.origin.x) > 0) d2 += d * d;
  else if ((d = s.origin.x - b.greater_corner.x) > 0) d2 += d * d;
  if ((d = b.lesser_corner.y - s.origin.y) > 0) d2 += d * d;
  else if ((d = s.origin.y - b.greater_corner.y) > 0) d2 += d * d;
  if ((d = b.lesser_corner.z - s.origin.z) > 0) d2 += d * d;
  else if ((d = s.origin.z - b.greater_corner.z) > 0) d2 += d * d;
  return d2;
}

template <typename T, typename T2>
inline bool intersect(const OrientedBox<T>& b, const Sphere<T2>& s) {
  return box_dist2(b, s) <= (double)s.radius * (double)s.radius;
}

template <typename T>
inline bool intersect(const Sphere<T>& a, const Sphere<T>& b) {
  double dx = a.origin.x - b.origin.x, dy = a.origin.y - b.origin.y, dz = a.origin.z - b.origin.z;
  double rr = (double)a.radius + (double)b.radius;
  return dx * dx + dy * dy + dz * dz <= rr * rr;
}

/* True when every corner of the box lies inside the sphere. */
template <typename T, typename T2>
inline bool contained(const OrientedBox<T>& b, const Sphere<T2>& s) {
  double d2 = 0.0, d1, d2b;
  d1 = s.origin.x - b.lesser_corner.x; d2b = b.greater_corner.x - s.origin.x;
  d1 = d1 * d1; d2b = d2b * d2b; d2 += d1 > d2b ? d1 : d2b;
  d1 = s.origin.y - b.lesser_corner.y; d2b = b.greater_corner.y - s.origin.y;
  d1 = d1 * d1; d2b = d2b * d2b; d2 += d1 > d2b ? d1 : d2b;
  d1 = s.origin.z - b.lesser_corner.z; d2b = b.greater_corner.z - s.origin.z;
  d1 = d1 * d1; d2b = d2b * d2b; d2 += d1 > d2b ? d1 : d2b;
  return d2 <= (double)s.radius * (double)s.radius;
}

}  // namespace Space

#endif
