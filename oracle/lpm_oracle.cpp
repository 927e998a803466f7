// lpm_oracle.cpp -- TEST INFRASTRUCTURE ONLY (the oracle).
//
// CPU restatement (C++17 + OpenMP) of the barotropic-vorticity (BVE) path of
// pbosler/lpmKokkos: mesh seeds and uniform tree refinement, spherical geometry,
// the Biot-Savart / Green's-function direct sums, the RK4 stepper (with the
// reference's face-vorticity quirk), initial conditions, error norms and the
// spherical-Poisson known-answer solve.  Each function cites the reference
// file:line it restates.  Expression order follows the reference so that the
// FP64 results agree with it to rounding of the (unpinned) Kokkos reduction order.
//
// Parity status: the reference cannot be built here (Kokkos/Trilinos, MPI and VTK
// are absent), so this restatement is pinned against the reference's recorded
// spherical-Poisson psi linf table (scripts/poissonOutput.py:6-30) and against the
// analytic known answers its tests use (RH54 psi=f/30, solid-body rotation,
// geometry asserts of tests/LpmGeometryUnitTests.cpp:146-165, mesh sizes and the
// 4*pi surface area).
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load
// this library.  The product path never calls it.
//
// Build: oracle/Makefile (g++ -O2 -fopenmp -ffp-contract=off -shared -fPIC).

#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>
#include <stdexcept>
#include <string>

namespace orc {

typedef double Real;
typedef int Index;
static constexpr Real PI = 3.1415926535897932384626433832795027975;  // src/LpmDefs.hpp:82
static constexpr Index NULL_IND = -1;                                  // src/LpmDefs.hpp:102

// ---------------------------------------------------------------------------
// Geometry: src/LpmGeometry.hpp:203-469 (SphereGeometry), src/LpmUtilities.hpp:15-46
// ---------------------------------------------------------------------------
struct V3 { Real v[3]; Real& operator[](int i) { return v[i]; } const Real& operator[](int i) const { return v[i]; } };

static inline Real dot(const V3& a, const V3& b) { return a[0]*b[0] + a[1]*b[1] + a[2]*b[2]; }  // :279-282
static inline V3 cross(const V3& a, const V3& b) {                                               // :291-296
  V3 c;
  c[0] = a[1]*b[2] - a[2]*b[1];
  c[1] = a[2]*b[0] - a[0]*b[2];
  c[2] = a[0]*b[1] - a[1]*b[0];
  return c;
}
static inline Real mag(const V3& v) { return std::sqrt(dot(v, v)); }                            // :343-354
static inline void scale(const Real a, V3& v) { v[0] *= a; v[1] *= a; v[2] *= a; }              // :267-271
static inline void normalize(V3& v) { scale(1.0/mag(v), v); }                                   // :361-363
static inline Real distance(const V3& a, const V3& b) {                                         // :371-376
  const V3 cp = cross(a, b);
  const Real dp = dot(a, b);
  return std::atan2(mag(cp), dp);
}
static inline V3 barycenter(const V3* cv, const int n) {                                        // :412-422
  V3 v; v[0] = 0.0; v[1] = 0.0; v[2] = 0.0;
  for (int i = 0; i < n; ++i) { v[0] += cv[i][0]; v[1] += cv[i][1]; v[2] += cv[i][2]; }
  scale(1.0/n, v);
  normalize(v);
  return v;
}
static inline V3 midpoint(const V3& a, const V3& b) {                                           // :430-436
  V3 v;
  v[0] = 0.5*(a[0] + b[0]);
  v[1] = 0.5*(a[1] + b[1]);
  v[2] = 0.5*(a[2] + b[2]);
  normalize(v);
  return v;
}
static inline Real triArea(const V3& a, const V3& b, const V3& c) {                             // :444-453
  const Real s1 = distance(a, b);
  const Real s2 = distance(b, c);
  const Real s3 = distance(c, a);
  const Real half_perim = 0.5*(s1 + s2 + s3);
  const Real zz = std::tan(0.5*half_perim) * std::tan(0.5*(half_perim-s1)) * std::tan(0.5*(half_perim-s2)) *
                  std::tan(0.5*(half_perim-s3));
  return 4*std::atan(std::sqrt(zz));
}
static inline Real polygonArea(const V3& ctr, const V3* verts, const int nverts) {              // :461-468
  Real ar = 0;
  for (int i = 0; i < nverts; ++i) ar += triArea(ctr, verts[i], verts[(i+1)%nverts]);
  return ar;
}
static inline Real atan4(const Real y, const Real x) {                                          // src/LpmUtilities.hpp:15-46
  Real result = 0.0;
  if (x == 0.0) {
    if (y > 0.0) result = 0.5*PI;
    else if (y < 0.0) result = 1.5*PI;
    else if (y == 0.0) result = 0.0;
  } else if (y == 0) {
    if (x > 0.0) result = 0.0;
    else if (x < 0.0) result = PI;
  } else {
    Real theta = std::atan2(std::abs(y), std::abs(x));
    if (x > 0.0 && y > 0.0) result = theta;
    else if (x < 0.0 && y > 0.0) result = PI - theta;
    else if (x < 0.0 && y < 0.0) result = PI + theta;
    else if (x > 0.0 && y < 0.0) result = 2.0*PI - theta;
  }
  return result;
}
static inline Real latitude(const V3& v) { return std::atan2(v[2], std::sqrt(v[0]*v[0] + v[1]*v[1])); }  // :217-219
static inline Real longitude(const V3& v) { return atan4(v[1], v[0]); }                                   // :226-228

// ---------------------------------------------------------------------------
// Mesh seeds: mesh_seeds/icosTriSphereSeed.dat and mesh_seeds/cubedSphereSeed.dat,
// read by MeshSeed::readfile (src/LpmMeshSeed.cpp:20-232).  The tables are the seed
// files' contents: coordinates (vertices then face centres), edges (orig, dest,
// left, right), face vertices and face edges.  They fix the index order of every
// refined mesh, so they are reproduced number for number.
// ---------------------------------------------------------------------------
static const Real ICOS_CRDS[32][3] = {
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
  {0.00000000000000000, 0.00000000000000000, -1.00000000000000000},
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
static const Index ICOS_EDGES[30][4] = {
  {0,1,0,4},{1,2,0,6},{2,0,0,1},{2,3,1,8},{0,3,2,1},{3,4,2,10},{4,0,2,3},{4,5,3,12},{5,0,3,4},{5,1,4,14},
  {1,6,5,14},{6,7,5,15},{7,1,5,6},{7,2,6,7},{7,8,7,16},{8,2,7,8},{8,3,8,9},{8,9,9,17},{3,9,10,9},{9,4,10,11},
  {9,10,11,18},{10,4,11,12},{10,5,12,13},{10,6,13,19},{6,5,13,14},{11,6,19,15},{11,7,15,16},{8,11,17,16},
  {11,9,17,18},{10,11,19,18}};
static const Index ICOS_FACEVERTS[20][3] = {
  {0,1,2},{0,2,3},{0,3,4},{0,4,5},{0,5,1},{1,6,7},{7,2,1},{2,7,8},{8,3,2},{3,8,9},
  {9,4,3},{4,9,10},{10,5,4},{5,10,6},{6,1,5},{11,7,6},{11,8,7},{11,9,8},{11,10,9},{11,6,10}};
static const Index ICOS_FACEEDGES[20][3] = {
  {0,1,2},{2,3,4},{4,5,6},{6,7,8},{8,9,0},{10,11,12},{13,1,12},{13,14,15},{16,3,15},{16,17,18},
  {19,5,18},{19,20,21},{22,7,21},{22,23,24},{10,9,24},{26,11,25},{27,14,26},{28,17,27},{29,20,28},{25,23,29}};

static const Real CUBE_CRDS[14][3] = {
  {0.57735026918962584, -0.57735026918962584, 0.57735026918962584},
  {0.57735026918962584, -0.57735026918962584, -0.57735026918962584},
  {0.57735026918962584, 0.57735026918962584, -0.57735026918962584},
  {0.57735026918962584, 0.57735026918962584, 0.57735026918962584},
  {-0.57735026918962584, 0.57735026918962584, -0.57735026918962584},
  {-0.57735026918962584, 0.57735026918962584, 0.57735026918962584},
  {-0.57735026918962584, -0.57735026918962584, -0.57735026918962584},
  {-0.57735026918962584, -0.57735026918962584, 0.57735026918962584},
  {1.00000000000000000, 0.00000000000000000, 0.00000000000000000},
  {0.00000000000000000, 1.00000000000000000, 0.00000000000000000},
  {-1.00000000000000000, 0.00000000000000000, 0.00000000000000000},
  {0.00000000000000000, -1.00000000000000000, 0.00000000000000000},
  {0.00000000000000000, 0.00000000000000000, 1.00000000000000000},
  {0.00000000000000000, 0.00000000000000000, -1.00000000000000000}};
static const Index CUBE_EDGES[12][4] = {
  {0,1,0,3},{1,2,0,5},{2,3,0,1},{3,0,0,4},{2,4,1,5},{4,5,1,2},{5,3,1,4},{4,6,2,5},{6,7,2,3},{7,5,2,4},
  {6,1,3,5},{0,7,3,4}};
static const Index CUBE_FACEVERTS[6][4] = {{0,1,2,3},{3,2,4,5},{5,4,6,7},{7,6,1,0},{7,0,3,5},{1,6,4,2}};
static const Index CUBE_FACEEDGES[6][4] = {{0,1,2,3},{2,4,5,6},{5,7,8,9},{8,10,0,11},{11,3,6,9},{10,7,4,1}};

// ---------------------------------------------------------------------------
// Tree mesh: Coords (src/LpmCoords.hpp:74-81 insertHost), Edges (src/LpmEdges.cpp:12-25
// insertHost, :55-84 divide), Faces (src/LpmFaces.cpp:9-27 insertHost, :43-63 initFromSeed,
// :115-248 TriFace divide, :250-382 QuadFace divide), PolyMesh2d::treeInit
// (src/LpmPolyMesh2d.cpp:10-17 seedInit, :31-44 treeInit).
// Only the physical coordinates are kept: the Lagrangian copies are identical at t=0.
// ---------------------------------------------------------------------------
struct Mesh {
  int nfv = 0;
  std::vector<V3> verts;        // physVerts.crds
  std::vector<V3> faceCrds;     // physFaces.crds
  // edges
  std::vector<Index> eo, ed, el, er, ek0, ek1;
  // faces
  std::vector<Index> fverts, fedges, fcenter, fkids0;
  std::vector<Real> farea;
  std::vector<unsigned char> fmask;
  std::vector<int> flevel;

  Index nedges() const { return (Index)eo.size(); }
  Index nfaces() const { return (Index)farea.size(); }
  bool edgeHasKids(Index e) const { return e < nedges() && ek0[e] > 0; }   // src/LpmEdges.hpp:241-244
  bool faceHasKids(Index f) const { return fkids0[f] > 0; }                 // src/LpmFaces.hpp:187-190

  void insertEdge(Index o, Index d, Index l, Index r) {                      // src/LpmEdges.cpp:12-25
    eo.push_back(o); ed.push_back(d); el.push_back(l); er.push_back(r); ek0.push_back(NULL_IND); ek1.push_back(NULL_IND);
  }
  void divideEdge(Index ind) {                                               // src/LpmEdges.cpp:55-84
    const Index crd_ins_pt = (Index)verts.size();
    const Index edge_ins_pt = nedges();
    const V3 a = verts[eo[ind]], b = verts[ed[ind]];
    verts.push_back(midpoint(a, b));
    const Index o = eo[ind], d = ed[ind], l = el[ind], r = er[ind];
    insertEdge(o, crd_ins_pt, l, r);
    insertEdge(crd_ins_pt, d, l, r);
    ek0[ind] = edge_ins_pt;
    ek1[ind] = edge_ins_pt + 1;
  }
  void insertFace(Index ctr, const Index* vi, const Index* ei, Index prt, Real ar) {  // src/LpmFaces.cpp:9-27
    for (int i = 0; i < nfv; ++i) { fverts.push_back(vi[i]); fedges.push_back(ei[i]); }
    fkids0.push_back(NULL_IND);
    fcenter.push_back(ctr);
    farea.push_back(ar);
    flevel.push_back(flevel[prt] + 1);
    fmask.push_back(0);
  }
};

static void seedInit(Mesh& m, int kind) {
  const bool icos = (kind == 0);
  const int nv = icos ? 12 : 8, nf = icos ? 20 : 6, ne = icos ? 30 : 12;
  m.nfv = icos ? 3 : 4;
  const Real (*crds)[3] = icos ? ICOS_CRDS : CUBE_CRDS;
  for (int i = 0; i < nv; ++i) { V3 v; v[0] = crds[i][0]; v[1] = crds[i][1]; v[2] = crds[i][2]; m.verts.push_back(v); }
  for (int i = 0; i < ne; ++i) {
    const Index* e = icos ? ICOS_EDGES[i] : CUBE_EDGES[i];
    m.insertEdge(e[0], e[1], e[2], e[3]);
  }
  for (int i = 0; i < nf; ++i) {                                             // src/LpmFaces.cpp:43-63
    const Index* fv = icos ? ICOS_FACEVERTS[i] : CUBE_FACEVERTS[i];
    const Index* fe = icos ? ICOS_FACEEDGES[i] : CUBE_FACEEDGES[i];
    V3 ctr; ctr[0] = crds[nv+i][0]; ctr[1] = crds[nv+i][1]; ctr[2] = crds[nv+i][2];
    V3 vc[4];
    for (int j = 0; j < m.nfv; ++j) vc[j] = m.verts[fv[j]];
    for (int j = 0; j < m.nfv; ++j) { m.fverts.push_back(fv[j]); m.fedges.push_back(fe[j]); }
    m.fcenter.push_back(i);
    m.farea.push_back(polygonArea(ctr, vc, m.nfv));                          // MeshSeed::faceArea, src/LpmMeshSeed.cpp:308-321
    m.fkids0.push_back(NULL_IND);
    m.flevel.push_back(0);
    m.fmask.push_back(0);
    m.faceCrds.push_back(ctr);
  }
}

// Shared part of both dividers: split each parent edge (or reuse its kids) and wire the
// child edges to the child faces (src/LpmFaces.cpp:149-177 and :286-313).
static Index splitSide(Mesh& m, Index faceInd, int i, int n, Index kidsBase, Index* NFE) {
  const Index parentEdge = m.fedges[faceInd*n + i];
  Index ek0, ek1;
  if (m.edgeHasKids(parentEdge)) { ek0 = m.ek0[parentEdge]; ek1 = m.ek1[parentEdge]; }
  else { ek0 = m.nedges(); ek1 = m.nedges() + 1; m.divideEdge(parentEdge); }
  const bool positive = (faceInd == m.el[parentEdge]);                       // Faces::edgeIsPositive
  if (positive) {
    NFE[i*n + i] = ek0; m.el[ek0] = kidsBase + i;
    NFE[((i+1)%n)*n + i] = ek1; m.el[ek1] = kidsBase + (i+1)%n;
  } else {
    NFE[i*n + i] = ek1; m.er[ek1] = kidsBase + i;
    NFE[((i+1)%n)*n + i] = ek0; m.er[ek0] = kidsBase + (i+1)%n;
  }
  return m.ed[ek0];                                                          // c1dest
}

static void finishDivide(Mesh& m, Index faceInd, const Index* NFV, const Index* NFE) {
  const int n = m.nfv;
  V3 ctr[4]; Real area[4];
  for (int i = 0; i < 4; ++i) {                                              // :222-234 / :355-367
    V3 vc[4];
    for (int j = 0; j < n; ++j) vc[j] = m.verts[NFV[i*n + j]];
    ctr[i] = barycenter(vc, n);
    area[i] = polygonArea(ctr[i], vc, n);
  }
  const Index crd_ins_pt = (Index)m.faceCrds.size();
  for (int i = 0; i < 4; ++i) {
    m.faceCrds.push_back(ctr[i]);
    m.insertFace(crd_ins_pt + i, NFV + i*n, NFE + i*n, faceInd, area[i]);
  }
  m.fkids0[faceInd] = (Index)m.farea.size() - 4;                              // setKidsHost (kid 0 marks "divided")
  m.farea[faceInd] = 0.0;
  m.fmask[faceInd] = 1;
}

static void divideTri(Mesh& m, Index faceInd) {                              // src/LpmFaces.cpp:115-248
  Index NFV[12], NFE[12];
  for (int k = 0; k < 12; ++k) { NFV[k] = NULL_IND; NFE[k] = NULL_IND; }
  const Index kidsBase = m.nfaces();
  for (int i = 0; i < 3; ++i) NFV[i*3 + i] = m.fverts[faceInd*3 + i];
  for (int i = 0; i < 3; ++i) {
    const Index c1dest = splitSide(m, faceInd, i, 3, kidsBase, NFE);
    if (i == 0) { NFV[0*3+1] = c1dest; NFV[1*3+0] = c1dest; NFV[3*3+2] = c1dest; }
    else if (i == 1) { NFV[1*3+2] = c1dest; NFV[2*3+1] = c1dest; NFV[3*3+0] = c1dest; }
    else { NFV[2*3+0] = c1dest; NFV[0*3+2] = c1dest; NFV[3*3+1] = c1dest; }
  }
  for (int k = 0; k < 12; ++k) if (NFV[k] == NULL_IND) throw std::logic_error("TriFace::divide error: vertex connectivity");
  const Index eip = m.nedges();                                              // :204-214
  for (int i = 0; i < 3; ++i) NFE[3*3 + i] = eip + i;
  NFE[0*3+1] = eip + 1; NFE[1*3+2] = eip + 2; NFE[2*3+0] = eip;
  m.insertEdge(NFV[2*3+1], NFV[2*3+0], kidsBase + 3, kidsBase + 2);
  m.insertEdge(NFV[0*3+2], NFV[0*3+1], kidsBase + 3, kidsBase + 0);
  m.insertEdge(NFV[1*3+0], NFV[1*3+2], kidsBase + 3, kidsBase + 1);
  finishDivide(m, faceInd, NFV, NFE);
}

static void divideQuad(Mesh& m, Index faceInd) {                             // src/LpmFaces.cpp:250-382
  Index NFV[16], NFE[16];
  for (int k = 0; k < 16; ++k) { NFV[k] = NULL_IND; NFE[k] = NULL_IND; }
  const Index kidsBase = m.nfaces();
  for (int i = 0; i < 4; ++i) NFV[i*4 + i] = m.fverts[faceInd*4 + i];
  for (int i = 0; i < 4; ++i) {
    const Index c1dest = splitSide(m, faceInd, i, 4, kidsBase, NFE);
    NFV[i*4 + (i+1)%4] = c1dest;
    NFV[((i+1)%4)*4 + i] = c1dest;
  }
  const Index bndry_insert_pt = (Index)m.verts.size();                       // :319-332 parent centre becomes a vertex
  m.verts.push_back(m.faceCrds[m.fcenter[faceInd]]);
  for (int i = 0; i < 4; ++i) NFV[i*4 + (i+2)%4] = bndry_insert_pt;
  const Index eip = m.nedges();                                              // :334-347
  m.insertEdge(NFV[0*4+1], NFV[0*4+2], kidsBase + 0, kidsBase + 1); NFE[0*4+1] = eip;     NFE[1*4+3] = eip;
  m.insertEdge(NFV[2*4+0], NFV[2*4+3], kidsBase + 3, kidsBase + 2); NFE[2*4+3] = eip + 1; NFE[3*4+1] = eip + 1;
  m.insertEdge(NFV[2*4+1], NFV[2*4+0], kidsBase + 1, kidsBase + 2); NFE[1*4+2] = eip + 2; NFE[2*4+0] = eip + 2;
  m.insertEdge(NFV[3*4+1], NFV[3*4+0], kidsBase + 0, kidsBase + 3); NFE[0*4+2] = eip + 3; NFE[3*4+0] = eip + 3;
  finishDivide(m, faceInd, NFV, NFE);
}

static void treeInit(Mesh& m, int kind, int depth) {                         // src/LpmPolyMesh2d.cpp:31-44
  seedInit(m, kind);
  for (int i = 0; i < depth; ++i) {
    const Index stopInd = m.nfaces();
    for (Index j = 0; j < stopInd; ++j) {
      if (!m.faceHasKids(j)) {
        if (kind == 0) divideTri(m, j); else divideQuad(m, j);
      }
    }
  }
}

// ---------------------------------------------------------------------------
// BVE pair kernels: src/LpmBVEKernels.hpp:21-26 (greensFn), :36-44 (biotSavart),
// reductions :49-102 (distinct: vertex targets) and :188-234 (collocated: face
// targets, i==j excluded by index).  eps is an option the reference lacks: the
// denominator becomes (1 - x.y + eps^2); eps = 0 gives the reference expressions.
// ---------------------------------------------------------------------------
static inline void biotSavart(Real u[3], const V3& tgt, const V3& src, Real vort, Real area, Real eps2) {
  const V3 c = cross(tgt, src);
  const Real strength = -vort * area / (4*PI*(1 - dot(src, tgt) + eps2));
  for (int j = 0; j < 3; ++j) u[j] = c[j] * strength;
}
static inline Real greensFn(const V3& tgt, const V3& src, Real vort, Real area, Real eps2) {
  const Real circ = -vort * area;
  return std::log(1 - dot(tgt, src) + eps2) * circ / (4*PI);
}

// One target: serial loop over sources (Kokkos TeamPolicy degenerates to this with team size 1).
static void reduceTarget(const V3& x, long self, const V3* sx, const Real* zeta, const Real* area,
                         const unsigned char* mask, long ns, Real eps2, Real u[3], Real* psi) {
  Real uu[3] = {0, 0, 0};
  Real pp = 0;
  for (long j = 0; j < ns; ++j) {
    if (mask[j] || j == self) continue;
    Real t[3];
    biotSavart(t, x, sx[j], zeta[j], area[j], eps2);
    uu[0] += t[0]; uu[1] += t[1]; uu[2] += t[2];
    if (psi) pp += greensFn(x, sx[j], zeta[j], area[j], eps2);
  }
  u[0] = uu[0]; u[1] = uu[1]; u[2] = uu[2];
  if (psi) *psi = pp;
}

static void velocityAll(const V3* vx, long nv, const V3* fx, const Real* zeta, const Real* area,
                        const unsigned char* mask, long nf, Real eps2, Real* vu, Real* fu, Real* vpsi, Real* fpsi) {
  #pragma omp parallel for schedule(dynamic, 64)
  for (long i = 0; i < nv + nf; ++i) {
    if (i < nv) reduceTarget(vx[i], -1, fx, zeta, area, mask, nf, eps2, vu + 3*i, vpsi ? vpsi + i : nullptr);
    else {
      const long k = i - nv;
      reduceTarget(fx[k], k, fx, zeta, area, mask, nf, eps2, fu + 3*k, fpsi ? fpsi + k : nullptr);
    }
  }
}

// ---------------------------------------------------------------------------
// Initial conditions: src/LpmRossbyWaves.hpp:18-53 (legendre54, SphHarm54, RH54Velocity),
// src/LpmVorticityGallery.hpp:25-40 (SolidBodyRotation).  Gaussian vortices are new
// (no reference class): zeta += a*exp(-(distance(x,c)/w)^2) with SphereGeometry::distance.
// ---------------------------------------------------------------------------
static inline Real legendre54(const Real z) { return z * (z*z - 1.0) * (z*z - 1.0); }
static inline Real sphHarm54(const V3& x) { const Real lam = longitude(x); return 30*std::cos(4*lam)*legendre54(x[2]); }
static inline void rh54Velocity(const V3& x, Real out[3]) {
  const Real theta = latitude(x);
  const Real lambda = longitude(x);
  const Real coslat = std::cos(theta), sinlat = std::sin(theta);
  const Real coslon = std::cos(lambda), sinlon = std::sin(lambda);
  const Real cl3 = coslat*coslat*coslat;                                      // cube(): src/LpmDefs.hpp
  const Real usph = 0.5*std::cos(4*lambda)*cl3*(5*std::cos(2*theta) - 3);
  const Real vsph = 4*cl3*sinlat*std::sin(4*lambda);
  out[0] = -usph*sinlon - vsph*sinlat*coslon;
  out[1] = usph*coslon - vsph*sinlat*sinlon;
  out[2] = vsph*coslat;
}

}  // namespace orc

using namespace orc;

extern "C" {

// ---------------------------------------------------------------------------
// Mesh export.  Arrays are malloc'd; free with oracle_mesh_free.
// ---------------------------------------------------------------------------
typedef struct {
  int kind, level;
  int nverts, nfaces, nleaves, nedges, nfv;
  double* vx;            // nverts*3, row-major
  double* fx;            // nfaces*3
  double* farea;         // nfaces
  unsigned char* fmask;  // nfaces
  int* flevel;           // nfaces
  int* fverts;           // nfaces*nfv
} oracle_mesh;

int oracle_mesh_build(int kind, int level, oracle_mesh* out) {
  if (!out || (kind != 0 && kind != 1) || level < 0 || level > 10) return -1;
  Mesh m;
  try { treeInit(m, kind, level); } catch (...) { return -2; }
  out->kind = kind; out->level = level;
  out->nverts = (int)m.verts.size(); out->nfaces = m.nfaces(); out->nedges = m.nedges(); out->nfv = m.nfv;
  int nl = 0; for (auto c : m.fmask) nl += (c == 0);
  out->nleaves = nl;
  out->vx = (double*)std::malloc(sizeof(double)*3*m.verts.size());
  out->fx = (double*)std::malloc(sizeof(double)*3*m.faceCrds.size());
  out->farea = (double*)std::malloc(sizeof(double)*m.farea.size());
  out->fmask = (unsigned char*)std::malloc(m.fmask.size());
  out->flevel = (int*)std::malloc(sizeof(int)*m.flevel.size());
  out->fverts = (int*)std::malloc(sizeof(int)*m.fverts.size());
  for (size_t i = 0; i < m.verts.size(); ++i) for (int c = 0; c < 3; ++c) out->vx[3*i+c] = m.verts[i][c];
  for (size_t i = 0; i < m.faceCrds.size(); ++i) for (int c = 0; c < 3; ++c) out->fx[3*i+c] = m.faceCrds[i][c];
  std::memcpy(out->farea, m.farea.data(), sizeof(double)*m.farea.size());
  std::memcpy(out->fmask, m.fmask.data(), m.fmask.size());
  std::memcpy(out->flevel, m.flevel.data(), sizeof(int)*m.flevel.size());
  std::memcpy(out->fverts, m.fverts.data(), sizeof(int)*m.fverts.size());
  return 0;
}

void oracle_mesh_free(oracle_mesh* m) {
  if (!m) return;
  std::free(m->vx); std::free(m->fx); std::free(m->farea); std::free(m->fmask); std::free(m->flevel); std::free(m->fverts);
  m->vx = m->fx = m->farea = nullptr; m->fmask = nullptr; m->flevel = m->fverts = nullptr;
}

// Geometry helpers exposed for the reference's geometry asserts (tests/LpmGeometryUnitTests.cpp:146-165).
double oracle_tri_area(const double* a, const double* b, const double* c) {
  V3 A, B, C; for (int i = 0; i < 3; ++i) { A[i] = a[i]; B[i] = b[i]; C[i] = c[i]; }
  return triArea(A, B, C);
}
void oracle_midpoint(const double* a, const double* b, double* out) {
  V3 A, B; for (int i = 0; i < 3; ++i) { A[i] = a[i]; B[i] = b[i]; }
  const V3 r = midpoint(A, B); for (int i = 0; i < 3; ++i) out[i] = r[i];
}
void oracle_barycenter(const double* pts, int n, double* out) {
  V3 v[8]; for (int k = 0; k < n && k < 8; ++k) for (int i = 0; i < 3; ++i) v[k][i] = pts[3*k+i];
  const V3 r = barycenter(v, n); for (int i = 0; i < 3; ++i) out[i] = r[i];
}
double oracle_polygon_area(const double* ctr, const double* pts, int n) {
  V3 c, v[8]; for (int i = 0; i < 3; ++i) c[i] = ctr[i];
  for (int k = 0; k < n && k < 8; ++k) for (int i = 0; i < 3; ++i) v[k][i] = pts[3*k+i];
  return polygonArea(c, v, n);
}
void oracle_cross(const double* a, const double* b, double* out) {
  V3 A, B; for (int i = 0; i < 3; ++i) { A[i] = a[i]; B[i] = b[i]; }
  const V3 r = cross(A, B); for (int i = 0; i < 3; ++i) out[i] = r[i];
}

// ---------------------------------------------------------------------------
// Direct sums (AoS row-major n*3 arrays).  vx may be null when nv == 0.
// BVEVertexVelocity / BVEVertexStreamFn (src/LpmBVEKernels.hpp:140-186) for vertices and
// BVEFaceVelocity / BVEFaceStreamFn (:263-305) for faces.
// ---------------------------------------------------------------------------
void oracle_bve_velocity(const double* vx, long nv, const double* fx, const double* zeta, const double* area,
                         const unsigned char* mask, long nf, double eps, double* vu, double* fu,
                         double* vpsi, double* fpsi) {
  velocityAll(reinterpret_cast<const V3*>(vx), nv, reinterpret_cast<const V3*>(fx), zeta, area, mask, nf,
              eps*eps, vu, fu, vpsi, fpsi);
}

// Distinct-set velocity for an arbitrary target list (no self exclusion): VelocityReduceDistinct.
void oracle_velocity_distinct(const double* tx, long nt, const double* sx, const double* zeta, const double* area,
                              const unsigned char* mask, long ns, double eps, double* u, double* psi) {
  const V3* T = reinterpret_cast<const V3*>(tx);
  const V3* S = reinterpret_cast<const V3*>(sx);
  const Real e2 = eps*eps;
  #pragma omp parallel for schedule(dynamic, 64)
  for (long i = 0; i < nt; ++i) reduceTarget(T[i], -1, S, zeta, area, mask, ns, e2, u + 3*i, psi ? psi + i : nullptr);
}

// Collocated sums at a subset of the faces: for each listed face index k the body of
// BVEFaceVelocity / BVEFaceStreamFn (src/LpmBVEKernels.hpp:263-305) -- every unmasked face j
// except j == k.  Each target of the reference's functor is independent of the others, so a
// subset gives the same values as the full launch at those faces.
void oracle_velocity_faces(const long* idx, long nt, const double* fx, const double* zeta, const double* area,
                           const unsigned char* mask, long nf, double eps, double* u, double* psi) {
  const V3* S = reinterpret_cast<const V3*>(fx);
  const Real e2 = eps*eps;
  #pragma omp parallel for schedule(dynamic, 16)
  for (long i = 0; i < nt; ++i)
    reduceTarget(S[idx[i]], idx[i], S, zeta, area, mask, nf, e2, u + 3*i, psi ? psi + i : nullptr);
}

// ---------------------------------------------------------------------------
// RK4: BVERK4::advance_timestep (src/LpmBVERK4_Impl.hpp:42-130) with BVERK4Update (:11-39),
// KokkosBlas::scal / update (x_k = dt*u; work = x + c*x_k) and BVEVorticityTendency
// (src/LpmBVEKernels.hpp:307-320).  quirk != 0 reproduces the face-vorticity update of
// :121 (facevort1, facevort2, facevort4, facevort4); quirk == 0 uses k3 as RK4 intends.
// renorm != 0 projects positions back to |x| = 1 after each step (an option; the reference has none).
// On entry vvel/fvel must hold u(x) (as left by init_vorticity or the previous step).
// ---------------------------------------------------------------------------
void oracle_bve_rk4(double* vx, double* vzeta, double* vvel, long nv,
                    double* fx, double* fzeta, double* fvel, const double* farea, const unsigned char* fmask, long nf,
                    double dt, double Omega, int nsteps, int quirk, int renorm, double eps) {
  std::vector<Real> vk[4], fk[4], vzk[4], fzk[4];
  for (int s = 0; s < 4; ++s) { vk[s].resize(3*nv); fk[s].resize(3*nf); vzk[s].resize(nv); fzk[s].resize(nf); }
  std::vector<Real> vxw(3*nv), fxw(3*nf), fzw(nf);
  const Real e2 = eps*eps;
  auto tend = [&](std::vector<Real>& dz, const double* vel, long n) {
    for (long i = 0; i < n; ++i) dz[i] = -2.0 * Omega * vel[3*i+2] * dt;
  };
  auto scal = [&](std::vector<Real>& xk, const double* vel, long n) {
    for (long i = 0; i < 3*n; ++i) xk[i] = dt * vel[i];
  };
  auto eval = [&](const Real* vxx, const Real* fxx, const Real* fz) {
    velocityAll(reinterpret_cast<const V3*>(vxx), nv, reinterpret_cast<const V3*>(fxx), fz, farea, fmask, nf, e2,
                vvel, fvel, nullptr, nullptr);
  };
  for (int step = 0; step < nsteps; ++step) {
    scal(vk[0], vvel, nv); tend(vzk[0], vvel, nv);                           // stage 1 (:63-68)
    scal(fk[0], fvel, nf); tend(fzk[0], fvel, nf);
    for (int s = 1; s < 4; ++s) {                                             // stages 2-4 (:70-116)
      const Real c = (s == 3) ? 1.0 : 0.5;
      for (long i = 0; i < 3*nv; ++i) vxw[i] = 1.0*vx[i] + c*vk[s-1][i];
      for (long i = 0; i < 3*nf; ++i) fxw[i] = 1.0*fx[i] + c*fk[s-1][i];
      for (long i = 0; i < nf; ++i) fzw[i] = 1.0*fzeta[i] + c*fzk[s-1][i];
      eval(vxw.data(), fxw.data(), fzw.data());
      scal(vk[s], vvel, nv); scal(fk[s], fvel, nf);
      tend(vzk[s], vvel, nv); tend(fzk[s], fvel, nf);
    }
    const Real sixth = 1.0/6.0, third = 1.0/3.0;                              // BVERK4Update (:11-39)
    for (long i = 0; i < nv; ++i) {
      for (int j = 0; j < 3; ++j)
        vx[3*i+j] += sixth*(vk[0][3*i+j] + vk[3][3*i+j]) + third*(vk[1][3*i+j] + vk[2][3*i+j]);
      vzeta[i] += sixth*(vzk[0][i] + vzk[3][i]) + third*(vzk[1][i] + vzk[2][i]);
    }
    const std::vector<Real>& fz3 = quirk ? fzk[3] : fzk[2];                  // (:121) quirk
    for (long i = 0; i < nf; ++i) {
      for (int j = 0; j < 3; ++j)
        fx[3*i+j] += sixth*(fk[0][3*i+j] + fk[3][3*i+j]) + third*(fk[1][3*i+j] + fk[2][3*i+j]);
      fzeta[i] += sixth*(fzk[0][i] + fzk[3][i]) + third*(fzk[1][i] + fz3[i]);
    }
    if (renorm) {
      for (long i = 0; i < nv; ++i) { V3 v; for (int j = 0; j < 3; ++j) v[j] = vx[3*i+j]; const Real r = mag(v);
        for (int j = 0; j < 3; ++j) vx[3*i+j] = v[j] / r; }
      for (long i = 0; i < nf; ++i) { V3 v; for (int j = 0; j < 3; ++j) v[j] = fx[3*i+j]; const Real r = mag(v);
        for (int j = 0; j < 3; ++j) fx[3*i+j] = v[j] / r; }
    }
    eval(vx, fx, fzeta);                                                      // RK4-0 (:123-126)
  }
}

// ---------------------------------------------------------------------------
// Initial conditions.
// ---------------------------------------------------------------------------
void oracle_ic_rh54(const double* x, long n, double* zeta) {                  // SphHarm54
  for (long i = 0; i < n; ++i) { V3 v; for (int j = 0; j < 3; ++j) v[j] = x[3*i+j]; zeta[i] = sphHarm54(v); }
}
void oracle_rh54_velocity(const double* x, long n, double* u) {               // RH54Velocity
  for (long i = 0; i < n; ++i) { V3 v; for (int j = 0; j < 3; ++j) v[j] = x[3*i+j]; rh54Velocity(v, u + 3*i); }
}
void oracle_ic_solid_body(const double* x, long n, double* zeta) {            // SolidBodyRotation::eval
  const Real OMEGA = 2*PI;
  for (long i = 0; i < n; ++i) zeta[i] = 2*OMEGA*x[3*i+2];
}
// Seeded Gaussian-vortex parameters (input generation, no reference counterpart):
// centres = normalised 3-vectors of Box-Muller normals, amplitudes U(lo, hi); uniforms are the
// top 53 bits of std::mt19937_64 draws.
void oracle_gaussian_params(unsigned long long seed, int ng, double lo, double hi, double* centers, double* amps) {
  std::mt19937_64 gen(seed);
  auto u53 = [&]() { return (double)(gen() >> 11) * (1.0 / 9007199254740992.0); };
  for (int g = 0; g < ng; ++g) {
    double v[3], r2 = 0.0;
    do {
      r2 = 0.0;
      for (int k = 0; k < 3; ++k) {
        const double a = 1.0 - u53();
        const double b = u53();
        v[k] = std::sqrt(-2.0*std::log(a)) * std::cos(2.0*PI*b);
        r2 += v[k]*v[k];
      }
    } while (r2 < 1e-20);
    const double sc = 1.0 / std::sqrt(r2);
    for (int k = 0; k < 3; ++k) centers[3*g+k] = v[k]*sc;
    amps[g] = lo + (hi - lo)*u53();
  }
}

void oracle_ic_gaussians_add(const double* x, long n, const double* centers, const double* amps, int ng,
                             double width, double* zeta) {
  for (long i = 0; i < n; ++i) {
    V3 v; for (int j = 0; j < 3; ++j) v[j] = x[3*i+j];
    Real z = zeta[i];
    for (int g = 0; g < ng; ++g) {
      V3 c; for (int j = 0; j < 3; ++j) c[j] = centers[3*g+j];
      const Real d = distance(v, c) / width;
      z += amps[g] * std::exp(-(d*d));
    }
    zeta[i] = z;
  }
}

// ---------------------------------------------------------------------------
// Area-weighted error norms, vector field: ErrNorms::compute (src/LpmErrorNorms.cpp:16-45).
// out = {l1, l2, linf}.
// ---------------------------------------------------------------------------
void oracle_errnorms_vec(const double* appx, const double* exact, const double* wt, long n, double* out) {
  Real l1n = 0, l1d = 0, l2n = 0, l2d = 0, lin = 0, lid = 0;
  for (long i = 0; i < n; ++i) {
    V3 e, x;
    for (int j = 0; j < 3; ++j) { e[j] = appx[3*i+j] - exact[3*i+j]; x[j] = exact[3*i+j]; }
    const Real em = mag(e), xm = mag(x);
    l1n += em*wt[i]; l1d += xm*wt[i]; l2n += em*em*wt[i]; l2d += xm*xm*wt[i];
    if (em > lin) lin = em;
    if (xm > lid) lid = xm;
  }
  out[0] = l1n/l1d; out[1] = std::sqrt(l2n/l2d); out[2] = lin/lid;
}

// ErrNorms::compute for scalars (src/LpmErrorNorms.cpp:47-70): l1/l2 of |e| and |exact|; linf is
// the largest SIGNED error over the largest signed exact value, starting from the max-reduction
// identity (the lowest double), as the reference's lambda writes it.
void oracle_errnorms_scalar(const double* appx, const double* exact, const double* wt, long n, double* out) {
  Real l1n = 0, l1d = 0, l2n = 0, l2d = 0, lin = -DBL_MAX, lid = -DBL_MAX;
  for (long i = 0; i < n; ++i) {
    const Real e = appx[i] - exact[i], x = exact[i];
    l1n += std::abs(e)*wt[i]; l1d += std::abs(x)*wt[i];
    l2n += e*e*wt[i]; l2d += x*x*wt[i];
    lin = e > lin ? e : lin;
    lid = x > lid ? x : lid;
  }
  out[0] = l1n/l1d; out[1] = std::sqrt(l2n/l2d); out[2] = lin/lid;
}

// Velocity tangency diagnostic: SphereVelocityTangentTestFunctor (src/LpmSphereTestKernels.hpp:11-25)
// with SphereGeometry::dot (src/LpmGeometry.hpp:280-282): udotx[i] = x0 u0 + x1 u1 + x2 u2.
void oracle_tangency(const double* x, const double* u, long n, double* udotx) {
  for (long i = 0; i < n; ++i) udotx[i] = x[3*i]*u[3*i] + x[3*i+1]*u[3*i+1] + x[3*i+2]*u[3*i+2];
}

// ---------------------------------------------------------------------------
// Spherical Poisson known-answer solve: SpherePoisson::init/solve (src/LpmSpherePoisson.hpp:419-475)
// with its own kernel spelling (:32-55): psi = -log(1 - x.y)*f*A/(4pi).  RH54 forcing,
// psi_exact = f/30, u_exact = RH54Velocity.  out = {mesh size [deg], linf psi verts,
// linf psi faces (leaves only), linf |u| verts, linf |u| faces (leaves only)}.
// ---------------------------------------------------------------------------
int oracle_poisson(int kind, int level, double* out) {
  Mesh m;
  try { treeInit(m, kind, level); } catch (...) { return -2; }
  const long nv = (long)m.verts.size(), nf = m.nfaces();
  std::vector<Real> fv(nv), ff(nf);
  for (long i = 0; i < nv; ++i) fv[i] = sphHarm54(m.verts[i]);
  for (long i = 0; i < nf; ++i) ff[i] = sphHarm54(m.faceCrds[i]);
  std::vector<Real> psiv(nv), psif(nf), uv(3*nv), uf(3*nf);
  auto solveOne = [&](const V3& x, long self, Real& psi, Real* u) {
    Real p = 0, uu[3] = {0, 0, 0};
    for (long j = 0; j < nf; ++j) {                                           // ReduceDistinct / ReduceCollocated
      if (m.fmask[j] || j == self) continue;
      p += -std::log(1.0 - dot(x, m.faceCrds[j]))*ff[j]*m.farea[j]/(4*PI);
    }
    for (long j = 0; j < nf; ++j) {                                           // UReduceDistinct / UReduceCollocated
      if (m.fmask[j] || j == self) continue;
      const V3 c = cross(x, m.faceCrds[j]);
      const Real str = -ff[j]*m.farea[j]/(4*PI*(1 - dot(x, m.faceCrds[j])));
      for (int k = 0; k < 3; ++k) uu[k] += c[k]*str;
    }
    psi = p; u[0] = uu[0]; u[1] = uu[1]; u[2] = uu[2];
  };
  #pragma omp parallel for schedule(dynamic, 16)
  for (long i = 0; i < nv + nf; ++i) {
    if (i < nv) solveOne(m.verts[i], -1, psiv[i], &uv[3*i]);
    else solveOne(m.faceCrds[i-nv], i-nv, psif[i-nv], &uf[3*(i-nv)]);
  }
  Real lv = 0, lf = 0, luv = 0, luf = 0;                                      // Error / UError (:273-352)
  for (long i = 0; i < nv; ++i) {
    const Real e = std::abs(psiv[i] - fv[i]/30.0); if (e > lv) lv = e;
    Real ue[3]; rh54Velocity(m.verts[i], ue);
    Real em = 0; for (int k = 0; k < 3; ++k) { const Real d = std::abs(uv[3*i+k] - ue[k]); em += d*d; }
    if (em > luv) luv = em;
  }
  for (long i = 0; i < nf; ++i) {
    if (m.fmask[i]) continue;
    const Real e = std::abs(psif[i] - ff[i]/30.0); if (e > lf) lf = e;
    Real ue[3]; rh54Velocity(m.faceCrds[i], ue);
    Real em = 0; for (int k = 0; k < 3; ++k) { const Real d = std::abs(uf[3*i+k] - ue[k]); em += d*d; }
    if (em > luf) luf = em;
  }
  int nl = 0; for (auto c : m.fmask) nl += (c == 0);
  out[0] = std::sqrt(4*PI/nl) * (180.0/PI);                                   // meshSize()*RAD2DEG
  out[1] = lv; out[2] = lf; out[3] = std::sqrt(luv); out[4] = std::sqrt(luf);
  return 0;
}

}  // extern "C"
