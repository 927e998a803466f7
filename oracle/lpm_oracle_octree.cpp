// lpm_oracle_octree.cpp -- TEST INFRASTRUCTURE ONLY (the oracle).
//
// Serial CPU restatement of the data-parallel Morton octree of pbosler/lpmKokkos
// (Zhou et al. 2011, listings 1 and 2), the reference that the GPU octree is compared with:
//
//   bounding box            BoxFunctor / BBoxReducer     src/LpmBox3d.hpp:84-160
//   cube from box           box2cube                     src/LpmBox3d.hpp:290-303
//   point keys              compute_key_for_point        src/LpmOctreeUtil.hpp:57-81
//   key algebra             parent_key / local_key / node_key   src/LpmOctreeUtil.hpp:83-135
//   codes, sort, permute    EncodeFunctor, ko::sort, PermuteFunctor
//                                                        src/LpmOctreeKernels.hpp:27-72,
//                                                        src/LpmNodeArrayD.cpp:14-58
//   unique leaf keys        MarkDuplicates, UniqueNodeFunctor   src/LpmOctreeKernels.hpp:99-183
//   full sibling sets       NodeSiblingCounter, NodeArrayDFunctor  :186-283
//   internal levels, root   ParentNodeFunctor, NodeArrayInternalFunctor :285-369,
//                           src/LpmNodeArrayInternal.cpp:13-186
//   concatenation           Tree::initNodes              src/LpmOctree.cpp:21-117
//   neighbours              NeighborhoodFunctor          src/LpmOctreeKernels.hpp:371-400
//
// Parents, kids and neighbours hold level-local indices, as the reference stores them.  One
// divergence: the reference's Tree::initNodes (src/LpmOctree.cpp:105-110) runs the
// neighbourhood walk over the concatenated arrays but reads the parent's neighbour row and the
// neighbour's kid row at the LEVEL-LOCAL index, which is the right row only at level 1.  Here
// those rows are read at base_address(l-1) + index, so every level holds the neighbours the
// construction defines (at level 1 both agree).
//
// The two neighbour lookup tables (src/LpmOctreeLUT.hpp:70-137) are generated from their
// geometric definition; tests compare them with the reference's tables.

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

namespace orc_octree {

typedef double Real;
typedef int Index;
typedef uint64_t Key;
static constexpr Index NULL_IND = -1;
static constexpr Real ZERO_TOL = 1.0e-14;  // src/LpmDefs.hpp:99
static constexpr int MAX_DEPTH = 10;       // MAX_OCTREE_DEPTH, src/LpmOctreeUtil.hpp:24-28

struct Box { Real xmin, xmax, ymin, ymax, zmin, zmax; };

static Real longestEdge(const Box& b) {
  const Real dx = b.xmax - b.xmin, dy = b.ymax - b.ymin, dz = b.zmax - b.zmin;
  return std::max(std::max(dx, dy), dz);
}
static Real shortestEdge(const Box& b) {
  const Real dx = b.xmax - b.xmin, dy = b.ymax - b.ymin, dz = b.zmax - b.zmin;
  return std::min(std::min(dx, dy), dz);
}
static Real aspect(const Box& b) { return longestEdge(b) / shortestEdge(b); }
static void centroid(Real& cx, Real& cy, Real& cz, const Box& b) {
  cx = 0.5 * (b.xmin + b.xmax);
  cy = 0.5 * (b.ymin + b.ymax);
  cz = 0.5 * (b.zmin + b.zmax);
}
static void toCube(Box& b) {
  if (std::abs(aspect(b) - 1.0) > ZERO_TOL) {
    const Real h = 0.5 * longestEdge(b);
    Real cx, cy, cz;
    centroid(cx, cy, cz, b);
    b = Box{cx - h, cx + h, cy - h, cy + h, cz - h, cz + h};
  }
}

static Key pow2(int k) { return Key(1) << k; }

static Key pointKey(const Real* p, int depth, Box bb) {
  if (std::abs(aspect(bb) - 1) > ZERO_TOL) toCube(bb);
  Real cx, cy, cz;
  centroid(cx, cy, cz, bb);
  Real half = 0.5 * (bb.xmax - bb.xmin);
  Key key = 0;
  const int nbits = 3 * depth;
  for (int i = 1; i <= depth; ++i) {
    half *= 0.5;
    const int b = nbits - 3 * i;
    const bool rz = p[2] >= cz, ry = p[1] >= cy, rx = p[0] >= cx;
    key += rz ? pow2(b) : 0;
    cz += rz ? half : -half;
    key += ry ? pow2(b + 1) : 0;
    cy += ry ? half : -half;
    key += rx ? pow2(b + 2) : 0;
    cx += rx ? half : -half;
  }
  return key;
}

// Ancestor of key k (a key at max_depth) at level lev-1: the top 3(lev-1) key bits.
static Key parentKey(Key k, int lev, int maxDepth) {
  const int pzb = 3 * maxDepth - 3 * (lev - 1);
  Key mask = 0;
  for (int i = 3 * maxDepth; i >= pzb; --i) mask += pow2(i);
  return k & mask;
}
static Key localKey(Key k, int lev, int maxDepth) {
  const int pzb = 3 * maxDepth - 3 * (lev - 1);
  return (k >> (pzb - 3)) & 7;
}
static Key nodeKey(Key pk, Key lk, int lev, int maxDepth) {
  const int pzb = 3 * maxDepth - 3 * (lev - 1);
  return pk + (lk << (pzb - 3));
}

// First index of key in the sorted array, or NULL_IND.
static Index findFirst(const std::vector<Key>& sorted, Key key) {
  auto it = std::lower_bound(sorted.begin(), sorted.end(), key);
  return (it != sorted.end() && *it == key) ? Index(it - sorted.begin()) : NULL_IND;
}

// Neighbour j = 9a + 3b + c of a node with local key i = 4x + 2y + z, offsets (a-1, b-1, c-1)
// along (x, y, z): the neighbour's parent is the parent's neighbour tParent[i][j]; the
// neighbour is that node's kid tChild[i][j].
static void makeTables(int tParent[8][27], int tChild[8][27]) {
  for (int i = 0; i < 8; ++i) {
    const int bit[3] = {(i >> 2) & 1, (i >> 1) & 1, i & 1};
    for (int j = 0; j < 27; ++j) {
      const int off[3] = {j / 9 - 1, (j / 3) % 3 - 1, j % 3 - 1};
      int pj = 0, cj = 0;
      for (int a = 0; a < 3; ++a) {
        const int s = bit[a] + off[a];     // -1, 0, 1, 2: child coordinate in the parent's frame
        const int pOff = s < 0 ? -1 : (s > 1 ? 1 : 0);
        pj = 3 * pj + (pOff + 1);
        cj = 2 * cj + (s - 2 * pOff);
      }
      tParent[i][j] = pj;
      tChild[i][j] = cj;
    }
  }
}

struct Level {
  std::vector<Key> keys;
  std::vector<Index> start, count, parent, kids;  // kids: 8 per node
};

struct Tree {
  Box box{};
  std::vector<Real> sorted;  // 3n
  std::vector<Index> origIds, ptInLeaf;
  std::vector<Level> levels;  // 0 .. depth
};

// Full sibling sets of the sorted unique keys at level lev (keys at max_depth resolution):
// returns the node count and, per unique key, the inclusive-scan value of NodeSiblingCounter.
static std::vector<Index> siblingScan(const std::vector<Key>& ukeys, int lev, int maxDepth) {
  std::vector<Index> ns(ukeys.size());
  Index ct = 0;
  for (size_t i = 0; i < ukeys.size(); ++i) {
    const bool newParent = i == 0 || parentKey(ukeys[i], lev, maxDepth) != parentKey(ukeys[i - 1], lev, maxDepth);
    ct += newParent ? 8 : 0;
    ns[i] = ct;
  }
  return ns;
}

static Tree build(const Real* x, long n, int depth) {
  Tree T;
  Box b{x[0], x[0], x[1], x[1], x[2], x[2]};
  for (long i = 0; i < n; ++i) {
    b.xmin = std::min(b.xmin, x[3 * i]); b.xmax = std::max(b.xmax, x[3 * i]);
    b.ymin = std::min(b.ymin, x[3 * i + 1]); b.ymax = std::max(b.ymax, x[3 * i + 1]);
    b.zmin = std::min(b.zmin, x[3 * i + 2]); b.zmax = std::max(b.zmax, x[3 * i + 2]);
  }
  T.box = b;
  std::vector<uint64_t> codes(n);
  for (long i = 0; i < n; ++i) codes[i] = (pointKey(x + 3 * i, depth, b) << 32) + uint64_t(i);
  std::sort(codes.begin(), codes.end());
  T.sorted.resize(3 * n);
  T.origIds.resize(n);
  T.ptInLeaf.assign(n, NULL_IND);
  for (long i = 0; i < n; ++i) {
    const long id = long(codes[i] & 0xffffffffu);
    T.origIds[i] = Index(id);
    for (int c = 0; c < 3; ++c) T.sorted[3 * i + c] = x[3 * id + c];
  }
  // unique leaf keys with their point ranges
  std::vector<Key> ukeys;
  std::vector<Index> ustart, ucount;
  for (long i = 0; i < n; ++i) {
    const Key k = codes[i] >> 32;
    if (i == 0 || k != (codes[i - 1] >> 32)) {
      ukeys.push_back(k);
      ustart.push_back(Index(i));
      ucount.push_back(0);
    }
    ucount.back() += 1;
  }
  T.levels.resize(depth + 1);
  {  // leaves (NodeArrayDFunctor)
    const std::vector<Index> ns = siblingScan(ukeys, depth, depth);
    Level& L = T.levels[depth];
    const Index nn = ns.back();
    L.keys.resize(nn); L.start.resize(nn); L.count.resize(nn);
    L.parent.assign(nn, NULL_IND);
    L.kids.assign(size_t(nn) * 8, NULL_IND);
    for (size_t i = 0; i < ukeys.size(); ++i) {
      if (i > 0 && ns[i] == ns[i - 1]) continue;
      const Index kid0 = ns[i] - 8;
      const Key pk = parentKey(ukeys[i], depth, depth);
      for (int j = 0; j < 8; ++j) {
        const Index nd = kid0 + j;
        L.keys[nd] = pk + Key(j);
        const Index f = findFirst(ukeys, pk + Key(j));
        if (f != NULL_IND) {
          L.start[nd] = ustart[f];
          L.count[nd] = ucount[f];
          for (Index k = ustart[f]; k < ustart[f] + ucount[f]; ++k) T.ptInLeaf[k] = nd;
        } else {
          L.start[nd] = NULL_IND;
          L.count[nd] = 0;
        }
      }
    }
  }
  for (int lev = depth - 1; lev >= 0; --lev) {
    Level& low = T.levels[lev + 1];
    Level& L = T.levels[lev];
    if (lev == 0) {  // root (NodeArrayInternal::initFromLower / initFromLeaves, level 0)
      L.keys.assign(1, 0);
      L.start.assign(1, 0);
      L.count.assign(1, 0);
      for (int i = 0; i < 8; ++i) L.count[0] += low.count[i];
      L.parent.assign(1, NULL_IND);
      L.kids.resize(8);
      for (int i = 0; i < 8; ++i) L.kids[i] = i;
      for (int i = 0; i < 8; ++i) low.parent[i] = 0;
      break;
    }
    // ParentNodeFunctor: one parent per group of 8 lower nodes
    const size_t np = low.keys.size() / 8;
    std::vector<Key> pkeys(np);
    std::vector<Index> pstart(np), pcount(np);
    for (size_t i = 0; i < np; ++i) {
      pkeys[i] = parentKey(low.keys[8 * i], lev + 1, depth);
      pcount[i] = 0;
      for (int j = 0; j < 8; ++j) pcount[i] += low.count[8 * i + j];
      for (int j = 0; j < 8; ++j)
        if (low.start[8 * i + j] != NULL_IND) { pstart[i] = low.start[8 * i + j]; break; }
    }
    const std::vector<Index> ns = siblingScan(pkeys, lev, depth);
    const Index nn = ns.back();
    L.keys.resize(nn); L.start.resize(nn); L.count.resize(nn);
    L.parent.assign(nn, NULL_IND);
    L.kids.assign(size_t(nn) * 8, NULL_IND);
    for (size_t i = 0; i < np; ++i) {  // NodeArrayInternalFunctor
      if (i > 0 && ns[i] == ns[i - 1]) continue;
      const Key pk = parentKey(pkeys[i], lev, depth);
      const Index kid0 = ns[i] - 8;
      for (int j = 0; j < 8; ++j) {
        const Index nd = kid0 + j;
        const Key k = nodeKey(pk, Key(j), lev, depth);
        L.keys[nd] = k;
        const Index f = findFirst(pkeys, k);
        if (f != NULL_IND) {
          L.start[nd] = pstart[f];
          L.count[nd] = pcount[f];
          const Index k0 = findFirst(low.keys, k);
          for (int c = 0; c < 8; ++c) {
            L.kids[size_t(nd) * 8 + c] = k0 + c;
            low.parent[k0 + c] = nd;
          }
        } else {
          L.start[nd] = NULL_IND;
          L.count[nd] = 0;
        }
      }
    }
  }
  return T;
}

}  // namespace orc_octree

using namespace orc_octree;

extern "C" {

// Node counts per level (depth + 1 entries); returns the total, or a negative value for an
// invalid depth or an empty point set.
long oracle_octree_counts(const double* x, long n, int depth, int* nnodes_per_level) {
  if (depth < 1 || depth > MAX_DEPTH || n <= 0) return -1;
  const Tree T = build(x, n, depth);
  long tot = 0;
  for (int l = 0; l <= depth; ++l) {
    nnodes_per_level[l] = int(T.levels[l].keys.size());
    tot += nnodes_per_level[l];
  }
  return tot;
}

// The concatenated tree of Tree::initNodes (levels 0..depth at base_address(l)):
// box6 = the reduced bounding box (xmin, xmax, ymin, ymax, zmin, zmax); keys (uint32);
// pt_inds (2 per node: first sorted point or -1, count); parents; kids (8 per node) and
// neighbors (27 per node) as level-local indices or -1; sorted_pts (3n, row-major); orig_ids;
// pt_in_leaf (level-local leaf index of each sorted point).
int oracle_octree_build(const double* x, long n, int depth, double* box6, int* base_address, int* nnodes_per_level,
                        uint32_t* keys, int* pt_inds, int* parents, int* kids, int* neighbors, double* sorted_pts,
                        int* orig_ids, int* pt_in_leaf) {
  if (depth < 1 || depth > MAX_DEPTH || n <= 0) return -1;
  const Tree T = build(x, n, depth);
  box6[0] = T.box.xmin; box6[1] = T.box.xmax; box6[2] = T.box.ymin;
  box6[3] = T.box.ymax; box6[4] = T.box.zmin; box6[5] = T.box.zmax;
  long base = 0;
  for (int l = 0; l <= depth; ++l) {
    const Level& L = T.levels[l];
    base_address[l] = int(base);
    nnodes_per_level[l] = int(L.keys.size());
    for (size_t i = 0; i < L.keys.size(); ++i) {
      const long g = base + long(i);
      keys[g] = uint32_t(L.keys[i]);
      pt_inds[2 * g] = L.start[i];
      pt_inds[2 * g + 1] = L.count[i];
      parents[g] = L.parent[i];
      for (int c = 0; c < 8; ++c) kids[8 * g + c] = L.kids[8 * i + c];
    }
    base += long(L.keys.size());
  }
  int tp[8][27], tc[8][27];
  makeTables(tp, tc);
  for (int j = 0; j < 27; ++j) neighbors[j] = j == 13 ? 0 : NULL_IND;
  for (int l = 1; l <= depth; ++l) {
    const long b = base_address[l], bp = base_address[l - 1];
    for (long t = 0; t < nnodes_per_level[l]; ++t) {
      const Index p = parents[b + t];
      const int i = int(localKey(keys[b + t], l, depth));
      for (int j = 0; j < 27; ++j) {
        const Index h = neighbors[27 * (bp + p) + tp[i][j]];
        neighbors[27 * (b + t) + j] = h != NULL_IND ? kids[8 * (bp + h) + tc[i][j]] : NULL_IND;
      }
    }
  }
  std::memcpy(sorted_pts, T.sorted.data(), sizeof(double) * 3 * size_t(n));
  std::memcpy(orig_ids, T.origIds.data(), sizeof(int) * size_t(n));
  std::memcpy(pt_in_leaf, T.ptInLeaf.data(), sizeof(int) * size_t(n));
  return 0;
}

// The two neighbour tables, 8 x 27 each, row-major.
void oracle_octree_tables(int* parent_table, int* child_table) {
  int tp[8][27], tc[8][27];
  makeTables(tp, tc);
  std::memcpy(parent_table, tp, sizeof(tp));
  std::memcpy(child_table, tc, sizeof(tc));
}

// Key algebra of src/LpmOctreeUtil.hpp for the key tests: op 0 = compute_key_for_point
// (a = point index into x, box = box6), 1 = parent_key(k, lev, maxd), 2 = local_key,
// 3 = node_key(k, lk, lev, maxd); box_from_key is oracle_octree_box.
uint64_t oracle_octree_key(int op, const double* x, const double* box6, uint64_t k, uint64_t lk, int lev, int maxd) {
  const Box b{box6[0], box6[1], box6[2], box6[3], box6[4], box6[5]};
  switch (op) {
    case 0: return pointKey(x, lev, b);
    case 1: return parentKey(k, lev, maxd);
    case 2: return localKey(k, lev, maxd);
    default: return nodeKey(k, lk, lev, maxd);
  }
}

// box_from_key (src/LpmOctreeUtil.hpp:106-122): the box of key k at level lev of a tree of
// depth maxd inside root box rbox.
void oracle_octree_box(uint64_t k, const double* rbox, int lev, int maxd, double* out6) {
  const Box rb{rbox[0], rbox[1], rbox[2], rbox[3], rbox[4], rbox[5]};
  Real cx, cy, cz;
  centroid(cx, cy, cz, rb);
  Real half = 0.5 * (rb.xmax - rb.xmin);
  for (int i = 1; i <= lev; ++i) {
    half *= 0.5;
    const Key l = localKey(k, i, maxd);
    cz += (l & 1) ? half : -half;
    cy += (l & 2) ? half : -half;
    cx += (l & 4) ? half : -half;
  }
  out6[0] = cx - half; out6[1] = cx + half; out6[2] = cy - half;
  out6[3] = cy + half; out6[4] = cz - half; out6[5] = cz + half;
}

}  // extern "C"
