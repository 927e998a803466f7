// mesh.cpp -- host-side tree mesh and initial conditions for the BVE path.
//
// The mesh is the input generator of the BVE path: icosahedral-triangle and cubed-sphere
// seeds refined uniformly, with the index order of pbosler/lpmKokkos's
// PolyMesh2d::treeInit (src/LpmPolyMesh2d.cpp:31-44): faces are visited in index order,
// each side is split at its spherical midpoint (Edges::divide, src/LpmEdges.cpp:55-84)
// unless a neighbour already split it, four children are appended, and the parent is
// masked with zero area (src/LpmFaces.cpp:115-382).  Keeping that order makes every
// array index identical to the reference's, so a caller's views line up one for one.
//
// Compiled with -ffp-contract=off so x86-64 and aarch64 hosts produce the same bits.

#include "lpm_bve.h"

#include <cmath>
#include <cstdint>
#include <cstring>
#include <exception>
#include <new>
#include <random>
#include <vector>

namespace lpm {
namespace {

constexpr double kPi = 3.1415926535897932384626433832795027975;

struct Vec3 { double x, y, z; };

// Spherical geometry with the reference's evaluation order (src/LpmGeometry.hpp:279-468).
inline double dot3(const Vec3& a, const Vec3& b) { return a.x*b.x + a.y*b.y + a.z*b.z; }
inline Vec3 cross3(const Vec3& a, const Vec3& b) {
  return Vec3{a.y*b.z - a.z*b.y, a.z*b.x - a.x*b.z, a.x*b.y - a.y*b.x};
}
inline Vec3 unit(Vec3 v) {
  const double s = 1.0 / std::sqrt(dot3(v, v));   // normalize(): scale by 1/|v|
  return Vec3{v.x*s, v.y*s, v.z*s};
}
inline double arc(const Vec3& a, const Vec3& b) {
  const Vec3 c = cross3(a, b);
  return std::atan2(std::sqrt(dot3(c, c)), dot3(a, b));
}
inline double sphTriArea(const Vec3& a, const Vec3& b, const Vec3& c) {   // L'Huilier's formula
  const double s1 = arc(a, b), s2 = arc(b, c), s3 = arc(c, a);
  const double h = 0.5*(s1 + s2 + s3);
  const double t = std::tan(0.5*h) * std::tan(0.5*(h - s1)) * std::tan(0.5*(h - s2)) * std::tan(0.5*(h - s3));
  return 4*std::atan(std::sqrt(t));
}
inline double sphPolyArea(const Vec3& ctr, const Vec3* v, int n) {
  double a = 0;
  for (int i = 0; i < n; ++i) a += sphTriArea(ctr, v[i], v[(i + 1) % n]);
  return a;
}
inline Vec3 sphCentroid(const Vec3* v, int n) {
  Vec3 s{0.0, 0.0, 0.0};
  for (int i = 0; i < n; ++i) { s.x += v[i].x; s.y += v[i].y; s.z += v[i].z; }
  const double r = 1.0 / n;
  return unit(Vec3{s.x*r, s.y*r, s.z*r});
}
inline Vec3 sphMidpoint(const Vec3& a, const Vec3& b) {
  return unit(Vec3{0.5*(a.x + b.x), 0.5*(a.y + b.y), 0.5*(a.z + b.z)});
}

// Seed data of mesh_seeds/icosTriSphereSeed.dat and mesh_seeds/cubedSphereSeed.dat: vertex
// coordinates, face-centre coordinates, edges (origin, destination, left face, right face),
// face vertices and face edges.  These tables define the index order of every refined mesh.
struct Seed {
  int nv, nf, ne, n;  // vertices, faces, edges, vertices per face
  const double (*vcrd)[3];
  const double (*fcrd)[3];
  const int (*edge)[4];
  const int* fvert;
  const int* fedge;
};

const double kIcoV[12][3] = {
  {0.00000000000000000, 0.00000000000000000, 1.00000000000000000},
  {0.72360679774997894, 0.52573111211913359, 0.44721359549995793},
  {-0.27639320225002101, 0.85065080835203988, 0.44721359549995793},
  {-0.89442719099991586, 0.00000000000000000, 0.44721359549995793},
  {-0.27639320225002101, -0.85065080835203988, 0.44721359549995793},
  {0.72360679774997894, -0.52573111211913359, 0.44721359549995793},
  {0.89442719099991586, 0.00000000000000000, -0.44721359549995793},
  {0.27639320225002101, 0.85065080835203988, -0.44721359549995793},
  {-0.72360679774997894, 0.52573111211913359, -0.44721359549995793},
  {-0.72360679774997894, -0.52573111211913359, -0.44721359549995793},
  {0.27639320225002101, -0.85065080835203988, -0.44721359549995793},
  {0.00000000000000000, 0.00000000000000000, -1.00000000000000000}};
const double kIcoF[20][3] = {
  {0.18759247408507992, 0.57735026918962584, 0.79465447229176622},
  {-0.49112347318842298, 0.35682208977308993, 0.79465447229176611},
  {-0.49112347318842298, -0.35682208977308993, 0.79465447229176611},
  {0.18759247408507992, -0.57735026918962584, 0.79465447229176622},
  {0.60706199820668627, 0.00000000000000000, 0.79465447229176622},
  {0.79465447229176611, 0.57735026918962573, -0.18759247408507990},
  {0.30353099910334314, 0.93417235896271567, 0.18759247408507992},
  {-0.30353099910334314, 0.93417235896271567, -0.18759247408507992},
  {-0.79465447229176611, 0.57735026918962573, 0.18759247408507990},
  {-0.98224694637684595, 0.00000000000000000, -0.18759247408507990},
  {-0.79465447229176611, -0.57735026918962573, 0.18759247408507990},
  {-0.30353099910334314, -0.93417235896271567, -0.18759247408507992},
  {0.30353099910334314, -0.93417235896271567, 0.18759247408507992},
  {0.79465447229176611, -0.57735026918962573, -0.18759247408507990},
  {0.98224694637684595, 0.00000000000000000, 0.18759247408507990},
  {0.49112347318842298, 0.35682208977308993, -0.79465447229176611},
  {-0.18759247408507992, 0.57735026918962584, -0.79465447229176622},
  {-0.60706199820668627, 0.00000000000000000, -0.79465447229176622},
  {-0.18759247408507992, -0.57735026918962584, -0.79465447229176622},
  {0.49112347318842298, -0.35682208977308993, -0.79465447229176611}};
const int kIcoE[30][4] = {
  {0,1,0,4},{1,2,0,6},{2,0,0,1},{2,3,1,8},{0,3,2,1},{3,4,2,10},{4,0,2,3},{4,5,3,12},{5,0,3,4},{5,1,4,14},
  {1,6,5,14},{6,7,5,15},{7,1,5,6},{7,2,6,7},{7,8,7,16},{8,2,7,8},{8,3,8,9},{8,9,9,17},{3,9,10,9},{9,4,10,11},
  {9,10,11,18},{10,4,11,12},{10,5,12,13},{10,6,13,19},{6,5,13,14},{11,6,19,15},{11,7,15,16},{8,11,17,16},
  {11,9,17,18},{10,11,19,18}};
const int kIcoFV[60] = {0,1,2, 0,2,3, 0,3,4, 0,4,5, 0,5,1, 1,6,7, 7,2,1, 2,7,8, 8,3,2, 3,8,9,
                        9,4,3, 4,9,10, 10,5,4, 5,10,6, 6,1,5, 11,7,6, 11,8,7, 11,9,8, 11,10,9, 11,6,10};
const int kIcoFE[60] = {0,1,2, 2,3,4, 4,5,6, 6,7,8, 8,9,0, 10,11,12, 13,1,12, 13,14,15, 16,3,15, 16,17,18,
                        19,5,18, 19,20,21, 22,7,21, 22,23,24, 10,9,24, 26,11,25, 27,14,26, 28,17,27, 29,20,28, 25,23,29};

const double kCubV[8][3] = {
  {0.57735026918962584, -0.57735026918962584, 0.57735026918962584},
  {0.57735026918962584, -0.57735026918962584, -0.57735026918962584},
  {0.57735026918962584, 0.57735026918962584, -0.57735026918962584},
  {0.57735026918962584, 0.57735026918962584, 0.57735026918962584},
  {-0.57735026918962584, 0.57735026918962584, -0.57735026918962584},
  {-0.57735026918962584, 0.57735026918962584, 0.57735026918962584},
  {-0.57735026918962584, -0.57735026918962584, -0.57735026918962584},
  {-0.57735026918962584, -0.57735026918962584, 0.57735026918962584}};
const double kCubF[6][3] = {{1.0, 0.0, 0.0}, {0.0, 1.0, 0.0}, {-1.0, 0.0, 0.0},
                            {0.0, -1.0, 0.0}, {0.0, 0.0, 1.0}, {0.0, 0.0, -1.0}};
const int kCubE[12][4] = {{0,1,0,3},{1,2,0,5},{2,3,0,1},{3,0,0,4},{2,4,1,5},{4,5,1,2},{5,3,1,4},{4,6,2,5},
                          {6,7,2,3},{7,5,2,4},{6,1,3,5},{0,7,3,4}};
const int kCubFV[24] = {0,1,2,3, 3,2,4,5, 5,4,6,7, 7,6,1,0, 7,0,3,5, 1,6,4,2};
const int kCubFE[24] = {0,1,2,3, 2,4,5,6, 5,7,8,9, 8,10,0,11, 11,3,6,9, 10,7,4,1};

const Seed kSeeds[2] = {
  {12, 20, 30, 3, kIcoV, kIcoF, kIcoE, kIcoFV, kIcoFE},
  {8, 6, 12, 4, kCubV, kCubF, kCubE, kCubFV, kCubFE}};

// Child-face connectivity of one division.  Corner child i owns parent vertex i; for
// triangles child 3 is the centre triangle, for quads the parent's centre becomes the
// shared vertex C.  Entries: 0..n-1 = parent corner P_k, 10+k = midpoint m_k of side k,
// 20 = centre vertex C.
const int kTriChild[4][3] = {{0, 10, 12}, {10, 1, 11}, {12, 11, 2}, {11, 12, 10}};
const int kQuadChild[4][4] = {{0, 10, 20, 13}, {10, 1, 11, 20}, {20, 11, 2, 12}, {13, 20, 12, 3}};
// Interior edges: {origin, destination, left child, right child}, same vertex coding,
// and the (child, slot) pairs each one fills.
const int kTriInner[3][4] = {{11, 12, 3, 2}, {12, 10, 3, 0}, {10, 11, 3, 1}};
const int kTriInnerSlots[3][2][2] = {{{3, 0}, {2, 0}}, {{3, 1}, {0, 1}}, {{3, 2}, {1, 2}}};
const int kQuadInner[4][4] = {{10, 20, 0, 1}, {20, 12, 3, 2}, {11, 20, 1, 2}, {20, 13, 0, 3}};
const int kQuadInnerSlots[4][2][2] = {{{0, 1}, {1, 3}}, {{2, 3}, {3, 1}}, {{1, 2}, {2, 0}}, {{0, 2}, {3, 0}}};

class TreeMesh {
 public:
  explicit TreeMesh(const Seed& s) : n_(s.n) {
    for (int i = 0; i < s.nv; ++i) vert_.push_back(Vec3{s.vcrd[i][0], s.vcrd[i][1], s.vcrd[i][2]});
    for (int e = 0; e < s.ne; ++e) addEdge(s.edge[e][0], s.edge[e][1], s.edge[e][2], s.edge[e][3]);
    for (int f = 0; f < s.nf; ++f) {
      const Vec3 c{s.fcrd[f][0], s.fcrd[f][1], s.fcrd[f][2]};
      Vec3 corner[4];
      for (int k = 0; k < n_; ++k) corner[k] = vert_[s.fvert[f*n_ + k]];
      addFace(c, &s.fvert[f*n_], &s.fedge[f*n_], sphPolyArea(c, corner, n_));
    }
  }

  void refine(int levels) {
    for (int l = 0; l < levels; ++l) {
      const int nf = (int)area_.size();
      for (int f = 0; f < nf; ++f)
        if (firstKid_[f] <= 0) divide(f);
    }
  }

  const std::vector<Vec3>& verts() const { return vert_; }
  const std::vector<Vec3>& centres() const { return ctr_; }
  const std::vector<double>& areas() const { return area_; }
  const std::vector<uint8_t>& masks() const { return mask_; }
  const std::vector<int>& faceVerts() const { return fv_; }  // n_ vertex indices per face
  int vertsPerFace() const { return n_; }

 private:
  int n_;
  std::vector<Vec3> vert_;
  std::vector<int> eo_, ed_, el_, er_, ekid_;     // edges: origin, destination, left, right, first child
  std::vector<Vec3> ctr_;                         // face centres (particles)
  std::vector<int> fv_, fe_, firstKid_;
  std::vector<double> area_;
  std::vector<uint8_t> mask_;

  void addEdge(int o, int d, int l, int r) {
    eo_.push_back(o); ed_.push_back(d); el_.push_back(l); er_.push_back(r); ekid_.push_back(-1);
  }
  void addFace(const Vec3& c, const int* v, const int* e, double a) {
    ctr_.push_back(c);
    fv_.insert(fv_.end(), v, v + n_);
    fe_.insert(fe_.end(), e, e + n_);
    firstKid_.push_back(-1);
    area_.push_back(a);
    mask_.push_back(0);
  }
  // Halves of edge e (origin half, destination half); splits it on first use.
  void halves(int e, int& h0, int& h1) {
    if (ekid_[e] <= 0) {
      const int mid = (int)vert_.size();
      const int first = (int)eo_.size();
      vert_.push_back(sphMidpoint(vert_[eo_[e]], vert_[ed_[e]]));
      const int o = eo_[e], d = ed_[e], l = el_[e], r = er_[e];
      addEdge(o, mid, l, r);
      addEdge(mid, d, l, r);
      ekid_[e] = first;
    }
    h0 = ekid_[e];
    h1 = ekid_[e] + 1;
  }

  void divide(int f) {
    const int n = n_;
    const int kid0 = (int)area_.size();
    int P[4], mid[4], C = -1;
    int slotEdge[4][4];
    for (int k = 0; k < n; ++k) P[k] = fv_[f*n + k];
    for (int k = 0; k < n; ++k) {
      const int e = fe_[f*n + k];
      int h0, h1;
      halves(e, h0, h1);
      const int next = (k + 1) % n;
      if (el_[e] == f) {            // side runs P_k -> P_{k+1}: origin half belongs to child k
        slotEdge[k][k] = h0;    el_[h0] = kid0 + k;
        slotEdge[next][k] = h1; el_[h1] = kid0 + next;
      } else {                      // side runs P_{k+1} -> P_k
        slotEdge[k][k] = h1;    er_[h1] = kid0 + k;
        slotEdge[next][k] = h0; er_[h0] = kid0 + next;
      }
      mid[k] = ed_[h0];
    }
    if (n == 4) {                   // the parent centre becomes the children's shared vertex
      C = (int)vert_.size();
      vert_.push_back(ctr_[f]);
    }
    auto vid = [&](int code) { return code < 10 ? P[code] : (code < 20 ? mid[code - 10] : C); };
    const int ninner = (n == 3) ? 3 : 4;
    const int firstInner = (int)eo_.size();
    for (int i = 0; i < ninner; ++i) {
      const int* t = (n == 3) ? kTriInner[i] : kQuadInner[i];
      const int (*slots)[2] = (n == 3) ? kTriInnerSlots[i] : kQuadInnerSlots[i];
      addEdge(vid(t[0]), vid(t[1]), kid0 + t[2], kid0 + t[3]);
      slotEdge[slots[0][0]][slots[0][1]] = firstInner + i;
      slotEdge[slots[1][0]][slots[1][1]] = firstInner + i;
    }
    Vec3 kc[4];
    double ka[4];
    int kv[4][4];
    for (int c = 0; c < 4; ++c) {
      Vec3 corner[4];
      for (int s = 0; s < n; ++s) {
        kv[c][s] = vid((n == 3) ? kTriChild[c][s] : kQuadChild[c][s]);
        corner[s] = vert_[kv[c][s]];
      }
      kc[c] = sphCentroid(corner, n);
      ka[c] = sphPolyArea(kc[c], corner, n);
    }
    for (int c = 0; c < 4; ++c) addFace(kc[c], kv[c], slotEdge[c], ka[c]);
    firstKid_[f] = kid0;
    area_[f] = 0.0;
    mask_[f] = 1;
  }
};

int64_t pow4(int l) { int64_t r = 1; for (int i = 0; i < l; ++i) r *= 4; return r; }

// atan2 with output range [0, 2 pi) (atan4, src/LpmUtilities.hpp:15-46).
double longitudeOf(double x, double y) {
  if (x == 0.0) { if (y > 0.0) return 0.5*kPi; if (y < 0.0) return 1.5*kPi; return 0.0; }
  if (y == 0.0) return x > 0.0 ? 0.0 : kPi;
  const double t = std::atan2(std::abs(y), std::abs(x));
  if (x > 0.0 && y > 0.0) return t;
  if (x < 0.0 && y > 0.0) return kPi - t;
  if (x < 0.0 && y < 0.0) return kPi + t;
  return 2.0*kPi - t;
}

// Portable uniform in [0,1) from the top 53 bits of a 64-bit draw.
inline double uniform53(std::mt19937_64& g) { return (double)(g() >> 11) * (1.0 / 9007199254740992.0); }

}  // namespace
}  // namespace lpm

extern "C" {

int lpm_mesh_counts(int seed, int level, int64_t* nverts, int64_t* nfaces, int64_t* nleaves) {
  if ((seed != LPM_SEED_ICOS_TRI && seed != LPM_SEED_CUBED) || level < 0 || level > 12) return LPM_ERR_INVALID_ARGUMENT;
  const int64_t f0 = seed == LPM_SEED_ICOS_TRI ? 20 : 6;
  const int64_t v0 = seed == LPM_SEED_ICOS_TRI ? 10 : 6;
  int64_t all = 0;
  for (int l = 0; l <= level; ++l) all += f0 * lpm::pow4(l);
  if (nverts) *nverts = 2 + v0 * lpm::pow4(level);
  if (nfaces) *nfaces = all;
  if (nleaves) *nleaves = f0 * lpm::pow4(level);
  return LPM_OK;
}

int lpm_mesh_build(int seed, int level, double* vx, double* fx, double* farea, uint8_t* fmask) {
  if ((seed != LPM_SEED_ICOS_TRI && seed != LPM_SEED_CUBED) || level < 0 || level > 10) return LPM_ERR_INVALID_ARGUMENT;
  try {
    lpm::TreeMesh m(lpm::kSeeds[seed]);
    m.refine(level);
    const auto& v = m.verts();
    const auto& c = m.centres();
    for (size_t i = 0; vx && i < v.size(); ++i) { vx[3*i] = v[i].x; vx[3*i+1] = v[i].y; vx[3*i+2] = v[i].z; }
    for (size_t i = 0; fx && i < c.size(); ++i) { fx[3*i] = c[i].x; fx[3*i+1] = c[i].y; fx[3*i+2] = c[i].z; }
    if (farea) std::memcpy(farea, m.areas().data(), sizeof(double) * m.areas().size());
    if (fmask) std::memcpy(fmask, m.masks().data(), m.masks().size());
  } catch (const std::bad_alloc&) {
    return LPM_ERR_OUT_OF_MEMORY;
  } catch (const std::exception&) {
    return LPM_ERR_INTERNAL;
  }
  return LPM_OK;
}

int lpm_mesh_face_verts(int seed, int level, int32_t* face_verts, int* verts_per_face) {
  if ((seed != LPM_SEED_ICOS_TRI && seed != LPM_SEED_CUBED) || level < 0 || level > 10) return LPM_ERR_INVALID_ARGUMENT;
  try {
    lpm::TreeMesh m(lpm::kSeeds[seed]);
    m.refine(level);
    if (verts_per_face) *verts_per_face = m.vertsPerFace();
    if (face_verts) std::memcpy(face_verts, m.faceVerts().data(), sizeof(int32_t) * m.faceVerts().size());
  } catch (const std::bad_alloc&) {
    return LPM_ERR_OUT_OF_MEMORY;
  } catch (const std::exception&) {
    return LPM_ERR_INTERNAL;
  }
  return LPM_OK;
}

int lpm_ic_rh54(const double* x, int64_t n, double* zeta) {
  if (n < 0 || (n > 0 && (!x || !zeta))) return LPM_ERR_INVALID_ARGUMENT;
  for (int64_t i = 0; i < n; ++i) {
    const double z = x[3*i+2];
    const double lam = lpm::longitudeOf(x[3*i], x[3*i+1]);
    zeta[i] = 30*std::cos(4*lam)*(z * (z*z - 1.0) * (z*z - 1.0));
  }
  return LPM_OK;
}

int lpm_ic_rh54_velocity(const double* x, int64_t n, double* u) {
  if (n < 0 || (n > 0 && (!x || !u))) return LPM_ERR_INVALID_ARGUMENT;
  for (int64_t i = 0; i < n; ++i) {
    const double px = x[3*i], py = x[3*i+1], pz = x[3*i+2];
    const double th = std::atan2(pz, std::sqrt(px*px + py*py));
    const double la = lpm::longitudeOf(px, py);
    const double cl = std::cos(th), sl = std::sin(th), co = std::cos(la), so = std::sin(la);
    const double cl3 = cl*cl*cl;
    const double us = 0.5*std::cos(4*la)*cl3*(5*std::cos(2*th) - 3);
    const double vs = 4*cl3*sl*std::sin(4*la);
    u[3*i] = -us*so - vs*sl*co;
    u[3*i+1] = us*co - vs*sl*so;
    u[3*i+2] = vs*cl;
  }
  return LPM_OK;
}

int lpm_ic_solid_body(const double* x, int64_t n, double* zeta) {
  if (n < 0 || (n > 0 && (!x || !zeta))) return LPM_ERR_INVALID_ARGUMENT;
  const double omega = 2*lpm::kPi;
  for (int64_t i = 0; i < n; ++i) zeta[i] = 2*omega*x[3*i+2];
  return LPM_OK;
}

int lpm_ic_gaussians_add(const double* x, int64_t n, const double* centers, const double* amps, int ng,
                         double width, double* zeta) {
  if (n < 0 || ng < 0 || !(width > 0) || (n > 0 && (!x || !zeta)) || (ng > 0 && (!centers || !amps)))
    return LPM_ERR_INVALID_ARGUMENT;
  for (int64_t i = 0; i < n; ++i) {
    const lpm::Vec3 p{x[3*i], x[3*i+1], x[3*i+2]};
    double z = zeta[i];
    for (int g = 0; g < ng; ++g) {
      const double d = lpm::arc(p, lpm::Vec3{centers[3*g], centers[3*g+1], centers[3*g+2]}) / width;
      z += amps[g] * std::exp(-(d*d));
    }
    zeta[i] = z;
  }
  return LPM_OK;
}

int lpm_ic_gaussian_params(uint64_t seed, int ng, double amp_lo, double amp_hi, double* centers, double* amps) {
  if (ng < 0 || (ng > 0 && (!centers || !amps))) return LPM_ERR_INVALID_ARGUMENT;
  std::mt19937_64 gen(seed);
  for (int g = 0; g < ng; ++g) {
    double v[3], r2 = 0.0;
    do {                                   // Box-Muller normals -> uniform direction on the sphere
      r2 = 0.0;
      for (int k = 0; k < 3; ++k) {
        const double u1 = 1.0 - lpm::uniform53(gen);   // (0, 1]
        const double u2 = lpm::uniform53(gen);
        v[k] = std::sqrt(-2.0*std::log(u1)) * std::cos(2.0*lpm::kPi*u2);
        r2 += v[k]*v[k];
      }
    } while (r2 < 1e-20);
    const double s = 1.0 / std::sqrt(r2);
    for (int k = 0; k < 3; ++k) centers[3*g+k] = v[k]*s;
    amps[g] = amp_lo + (amp_hi - amp_lo)*lpm::uniform53(gen);
  }
  return LPM_OK;
}

}  // extern "C"
