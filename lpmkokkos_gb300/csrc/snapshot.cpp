// snapshot.cpp -- checkpoint / restart of a BVE state and legacy-VTK output
// (include/lpm_bve_snapshot.h).
//
// Snapshot file (little-endian, this library's own format):
//   header, 128 bytes: char magic[8] = "LPMBVE01"; int32 version (1); int32 seed; int32 level;
//     int32 verts_per_face (0 = unknown); int64 nverts; int64 nfaces; double t; double dt;
//     double omega; padding to 128 bytes
//   then, row-major float64 unless noted: vx (nverts x 3), vzeta (nverts), vvel (nverts x 3),
//     fx (nfaces x 3), fzeta (nfaces), fvel (nfaces x 3), farea (nfaces), fmask (nfaces bytes)
// Every array of lpm_bve_state is saved and restored bit for bit.  A run stepped on from a
// restored state builds a new plan whose target/source order follows the restored positions,
// so it sums in another order than the uninterrupted run: the two agree to that rounding.
//
// VTK: legacy PolyData ("vtk DataFile Version 3.0", BINARY, big-endian as the format requires):
// POINTS = vertex positions, POLYGONS = leaf faces (mask 0) by their vertices, POINT_DATA
// relVort + velocity at vertices, CELL_DATA relVort, velocity and area of the leaf faces --
// the fields the reference's BVE driver adds before vtk.write (tests/LpmBVETest.cpp:98-106).

#include "lpm_bve_snapshot.h"
#include "engine_core.hpp"

#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

namespace lpm {
namespace {

constexpr char kMagic[8] = {'L', 'P', 'M', 'B', 'V', 'E', '0', '1'};
constexpr int kVersion = 1;

struct Header {
  char magic[8];
  int32_t version, seed, level, vpf;
  int64_t nverts, nfaces;
  double t, dt, omega;
  char pad[128 - 8 - 16 - 16 - 24];
};
static_assert(sizeof(Header) == 128, "snapshot header is 128 bytes");

bool littleEndian() {
  const uint16_t one = 1;
  uint8_t b;
  std::memcpy(&b, &one, 1);
  return b == 1;
}

struct File {
  std::FILE* f = nullptr;
  ~File() {
    if (f) std::fclose(f);
  }
};

// True for device or managed memory; false for host memory and whenever no CUDA device is
// present (the attribute query then fails and its error is cleared).
bool cudaOwned(const void* p) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    (void)cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

bool haveDevice() {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    (void)cudaGetLastError();
    return false;
  }
  return n > 0;
}

// Copies between the caller's arrays and host buffers.  Device or managed memory goes through
// `s`; host-only copies use memcpy (no device needed), after synchronising `s` when a device
// exists, so work queued on `s` into pinned host arrays is complete first.
void copyBytes(void* dst, const void* src, size_t bytes, cudaStream_t s) {
  if (bytes == 0) return;
  if (cudaOwned(dst) || cudaOwned(src)) {
    LPM_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, s));
    LPM_CUDA(cudaStreamSynchronize(s));
    return;
  }
  if (haveDevice()) LPM_CUDA(cudaStreamSynchronize(s));
  std::memcpy(dst, src, bytes);
}

// Strided n x 3 array (device or host) -> host row-major.
std::vector<double> fetchVec(const double* p, int64_t n, int64_t si, int64_t sc, cudaStream_t s) {
  std::vector<double> out(3 * (size_t)n);
  if (n == 0) return out;
  const int64_t span = (n - 1) * si + 2 * sc + 1;
  std::vector<double> raw((size_t)span);
  copyBytes(raw.data(), p, sizeof(double) * span, s);
  for (int64_t i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) out[3 * i + c] = raw[(size_t)(i * si + c * sc)];
  return out;
}

template <typename T>
std::vector<T> fetchScalar(const T* p, int64_t n, cudaStream_t s) {
  std::vector<T> out((size_t)n);
  if (n > 0) copyBytes(out.data(), p, sizeof(T) * n, s);
  return out;
}

// Host row-major n x 3 -> strided device (or host) array; the strided span is read first so
// that entries between the strides are kept.
void storeVec(double* p, const std::vector<double>& v, int64_t n, int64_t si, int64_t sc, cudaStream_t s) {
  if (n == 0) return;
  if (si == 3 && sc == 1) {
    copyBytes(p, v.data(), sizeof(double) * 3 * n, s);
    return;
  }
  const int64_t span = (n - 1) * si + 2 * sc + 1;
  std::vector<double> raw((size_t)span);
  copyBytes(raw.data(), p, sizeof(double) * span, s);
  for (int64_t i = 0; i < n; ++i)
    for (int c = 0; c < 3; ++c) raw[(size_t)(i * si + c * sc)] = v[3 * i + c];
  copyBytes(p, raw.data(), sizeof(double) * span, s);
}

template <typename T>
void storeScalar(T* p, const std::vector<T>& v, cudaStream_t s) {
  if (!v.empty()) copyBytes(p, v.data(), sizeof(T) * v.size(), s);
}

void checkState(const lpm_bve_state* st) {
  if (!st) fail(LPM_ERR_INVALID_ARGUMENT, "null state");
  checkVec("vx", st->vx, st->nverts, st->vx_stride_i, st->vx_stride_c);
  checkVec("vvel", st->vvel, st->nverts, st->vvel_stride_i, st->vvel_stride_c);
  checkVec("fx", st->fx, st->nfaces, st->fx_stride_i, st->fx_stride_c);
  checkVec("fvel", st->fvel, st->nfaces, st->fvel_stride_i, st->fvel_stride_c);
  if (st->nverts > 0 && !st->vzeta) fail(LPM_ERR_INVALID_ARGUMENT, "null vzeta");
  if (st->nfaces > 0 && (!st->fzeta || !st->farea)) fail(LPM_ERR_INVALID_ARGUMENT, "null fzeta/farea");
}

void writeAll(std::FILE* f, const void* p, size_t bytes, const char* path) {
  if (bytes && std::fwrite(p, 1, bytes, f) != bytes) fail(LPM_ERR_INVALID_ARGUMENT, "%s: write failed", path);
}
void readAll(std::FILE* f, void* p, size_t bytes, const char* path) {
  if (bytes && std::fread(p, 1, bytes, f) != bytes) fail(LPM_ERR_INVALID_ARGUMENT, "%s: truncated snapshot", path);
}

Header readHeader(std::FILE* f, const char* path) {
  Header h{};
  readAll(f, &h, sizeof(h), path);
  if (std::memcmp(h.magic, kMagic, 8) != 0) fail(LPM_ERR_INVALID_ARGUMENT, "%s: not a BVE snapshot", path);
  if (h.version != kVersion) fail(LPM_ERR_NOT_SUPPORTED, "%s: snapshot version %d", path, h.version);
  if (h.nverts < 0 || h.nfaces < 0) fail(LPM_ERR_INVALID_ARGUMENT, "%s: corrupt header", path);
  return h;
}

// Big-endian copy of a float64 / int32 array for legacy VTK binary sections.
template <typename T>
void writeBigEndian(std::FILE* f, const T* v, size_t n, const char* path) {
  std::vector<unsigned char> buf(n * sizeof(T));
  const bool swap = littleEndian();
  for (size_t i = 0; i < n; ++i) {
    unsigned char b[sizeof(T)];
    std::memcpy(b, &v[i], sizeof(T));
    for (size_t k = 0; k < sizeof(T); ++k) buf[i * sizeof(T) + k] = swap ? b[sizeof(T) - 1 - k] : b[k];
  }
  writeAll(f, buf.data(), buf.size(), path);
}

int fail_code(const Error& e, std::string* err) {
  if (err) *err = e.msg;
  std::fprintf(stderr, "lpm_bve snapshot: %s\n", e.msg.c_str());
  return e.code;
}

}  // namespace

// Shared by the C ABI below and the server: writes host row-major arrays.
void writeSnapshotHost(const char* path, int seed, int level, int vpf, int64_t nv, int64_t nf, double t, double dt,
                       double omega, const double* vx, const double* vzeta, const double* vvel, const double* fx,
                       const double* fzeta, const double* fvel, const double* farea, const uint8_t* fmask) {
  if (!littleEndian()) fail(LPM_ERR_NOT_SUPPORTED, "snapshots are written on little-endian hosts only");
  File F;
  F.f = std::fopen(path, "wb");
  if (!F.f) fail(LPM_ERR_INVALID_ARGUMENT, "%s: cannot open for writing", path);
  Header h{};
  std::memcpy(h.magic, kMagic, 8);
  h.version = kVersion;
  h.seed = seed;
  h.level = level;
  h.vpf = vpf;
  h.nverts = nv;
  h.nfaces = nf;
  h.t = t;
  h.dt = dt;
  h.omega = omega;
  writeAll(F.f, &h, sizeof(h), path);
  writeAll(F.f, vx, sizeof(double) * 3 * nv, path);
  writeAll(F.f, vzeta, sizeof(double) * nv, path);
  writeAll(F.f, vvel, sizeof(double) * 3 * nv, path);
  writeAll(F.f, fx, sizeof(double) * 3 * nf, path);
  writeAll(F.f, fzeta, sizeof(double) * nf, path);
  writeAll(F.f, fvel, sizeof(double) * 3 * nf, path);
  writeAll(F.f, farea, sizeof(double) * nf, path);
  std::vector<uint8_t> zeros;
  if (!fmask) zeros.assign((size_t)nf, 0);
  writeAll(F.f, fmask ? fmask : zeros.data(), (size_t)nf, path);
  if (std::fflush(F.f) != 0) fail(LPM_ERR_INVALID_ARGUMENT, "%s: write failed", path);
}

}  // namespace lpm

using namespace lpm;

extern "C" {

int lpm_bve_snapshot_write(const char* path, const lpm_bve_state* st, int seed, int level, double t, double dt,
                           double omega, lpm_stream_t stream) {
  try {
    if (!path) fail(LPM_ERR_INVALID_ARGUMENT, "null path");
    checkState(st);
    cudaStream_t s = (cudaStream_t)stream;
    const int64_t nv = st->nverts, nf = st->nfaces;
    const auto vx = fetchVec(st->vx, nv, st->vx_stride_i, st->vx_stride_c, s);
    const auto vv = fetchVec(st->vvel, nv, st->vvel_stride_i, st->vvel_stride_c, s);
    const auto fx = fetchVec(st->fx, nf, st->fx_stride_i, st->fx_stride_c, s);
    const auto fv = fetchVec(st->fvel, nf, st->fvel_stride_i, st->fvel_stride_c, s);
    const auto vz = fetchScalar(st->vzeta, nv, s);
    const auto fz = fetchScalar(st->fzeta, nf, s);
    const auto fa = fetchScalar(st->farea, nf, s);
    const auto fm = st->fmask ? fetchScalar(st->fmask, nf, s) : std::vector<uint8_t>((size_t)nf, 0);
    int vpf = 0;
    if (lpm_mesh_face_verts(seed, level, nullptr, &vpf) != LPM_OK) vpf = 0;
    writeSnapshotHost(path, seed, level, vpf, nv, nf, t, dt, omega, vx.data(), vz.data(), vv.data(), fx.data(),
                      fz.data(), fv.data(), fa.data(), fm.data());
  } catch (const Error& e) {
    return fail_code(e, nullptr);
  } catch (const std::exception& e) {
    return fail_code(fromStd(e), nullptr);
  }
  return LPM_OK;
}

int lpm_bve_snapshot_info(const char* path, int* seed, int* level, int64_t* nverts, int64_t* nfaces, double* t,
                          double* dt, double* omega) {
  try {
    if (!path) fail(LPM_ERR_INVALID_ARGUMENT, "null path");
    File F;
    F.f = std::fopen(path, "rb");
    if (!F.f) fail(LPM_ERR_INVALID_ARGUMENT, "%s: cannot open", path);
    const Header h = readHeader(F.f, path);
    if (seed) *seed = h.seed;
    if (level) *level = h.level;
    if (nverts) *nverts = h.nverts;
    if (nfaces) *nfaces = h.nfaces;
    if (t) *t = h.t;
    if (dt) *dt = h.dt;
    if (omega) *omega = h.omega;
  } catch (const Error& e) {
    return fail_code(e, nullptr);
  } catch (const std::exception& e) {
    return fail_code(fromStd(e), nullptr);
  }
  return LPM_OK;
}

int lpm_bve_snapshot_read(const char* path, const lpm_bve_state* st, double* t, lpm_stream_t stream) {
  try {
    if (!path) fail(LPM_ERR_INVALID_ARGUMENT, "null path");
    checkState(st);
    cudaStream_t s = (cudaStream_t)stream;
    File F;
    F.f = std::fopen(path, "rb");
    if (!F.f) fail(LPM_ERR_INVALID_ARGUMENT, "%s: cannot open", path);
    const Header h = readHeader(F.f, path);
    if (h.nverts != st->nverts || h.nfaces != st->nfaces)
      fail(LPM_ERR_INVALID_ARGUMENT, "%s: snapshot holds %lld vertices / %lld faces, the state %lld / %lld", path,
           (long long)h.nverts, (long long)h.nfaces, (long long)st->nverts, (long long)st->nfaces);
    const int64_t nv = h.nverts, nf = h.nfaces;
    std::vector<double> vx(3 * nv), vz(nv), vv(3 * nv), fx(3 * nf), fz(nf), fv(3 * nf), fa(nf);
    std::vector<uint8_t> fm(nf);
    readAll(F.f, vx.data(), sizeof(double) * vx.size(), path);
    readAll(F.f, vz.data(), sizeof(double) * vz.size(), path);
    readAll(F.f, vv.data(), sizeof(double) * vv.size(), path);
    readAll(F.f, fx.data(), sizeof(double) * fx.size(), path);
    readAll(F.f, fz.data(), sizeof(double) * fz.size(), path);
    readAll(F.f, fv.data(), sizeof(double) * fv.size(), path);
    readAll(F.f, fa.data(), sizeof(double) * fa.size(), path);
    readAll(F.f, fm.data(), fm.size(), path);
    // Areas and mask are mesh data the stepper only reads: they must already match.
    const auto myArea = fetchScalar(st->farea, nf, s);
    const auto myMask = st->fmask ? fetchScalar(st->fmask, nf, s) : std::vector<uint8_t>((size_t)nf, 0);
    if (std::memcmp(myArea.data(), fa.data(), sizeof(double) * nf) != 0 || myMask != fm)
      fail(LPM_ERR_INVALID_ARGUMENT, "%s: face areas or mask differ from the state's (another mesh)", path);
    storeVec(st->vx, vx, nv, st->vx_stride_i, st->vx_stride_c, s);
    storeVec(st->vvel, vv, nv, st->vvel_stride_i, st->vvel_stride_c, s);
    storeVec(st->fx, fx, nf, st->fx_stride_i, st->fx_stride_c, s);
    storeVec(st->fvel, fv, nf, st->fvel_stride_i, st->fvel_stride_c, s);
    storeScalar(st->vzeta, vz, s);
    storeScalar(st->fzeta, fz, s);
    if (t) *t = h.t;
  } catch (const Error& e) {
    return fail_code(e, nullptr);
  } catch (const std::exception& e) {
    return fail_code(fromStd(e), nullptr);
  }
  return LPM_OK;
}

int lpm_bve_vtk_write(const char* path, const lpm_bve_state* st, int seed, int level, lpm_stream_t stream) {
  try {
    if (!path) fail(LPM_ERR_INVALID_ARGUMENT, "null path");
    checkState(st);
    int64_t nv = 0, nf = 0, nl = 0;
    if (lpm_mesh_counts(seed, level, &nv, &nf, &nl) != LPM_OK)
      fail(LPM_ERR_INVALID_ARGUMENT, "vtk: mesh seed %d level %d", seed, level);
    if (nv != st->nverts || nf != st->nfaces)
      fail(LPM_ERR_INVALID_ARGUMENT, "vtk: state sizes do not match mesh seed %d level %d", seed, level);
    int vpf = 0;
    std::vector<int32_t> conn;
    lpm_mesh_face_verts(seed, level, nullptr, &vpf);
    conn.resize((size_t)nf * vpf);
    lpm_mesh_face_verts(seed, level, conn.data(), &vpf);
    cudaStream_t s = (cudaStream_t)stream;
    const auto vx = fetchVec(st->vx, nv, st->vx_stride_i, st->vx_stride_c, s);
    const auto vv = fetchVec(st->vvel, nv, st->vvel_stride_i, st->vvel_stride_c, s);
    const auto fv = fetchVec(st->fvel, nf, st->fvel_stride_i, st->fvel_stride_c, s);
    const auto vz = fetchScalar(st->vzeta, nv, s);
    const auto fz = fetchScalar(st->fzeta, nf, s);
    const auto fa = fetchScalar(st->farea, nf, s);
    const auto fm = st->fmask ? fetchScalar(st->fmask, nf, s) : std::vector<uint8_t>((size_t)nf, 0);
    std::vector<int64_t> leaves;
    for (int64_t f = 0; f < nf; ++f)
      if (!fm[f]) leaves.push_back(f);
    File F;
    F.f = std::fopen(path, "wb");
    if (!F.f) fail(LPM_ERR_INVALID_ARGUMENT, "%s: cannot open for writing", path);
    char line[256];
    auto put = [&](const char* text) { writeAll(F.f, text, std::strlen(text), path); };
    put("# vtk DataFile Version 3.0\nLPM BVE state\nBINARY\nDATASET POLYDATA\n");
    std::snprintf(line, sizeof(line), "POINTS %lld double\n", (long long)nv);
    put(line);
    writeBigEndian(F.f, vx.data(), vx.size(), path);
    const int64_t nl2 = (int64_t)leaves.size();
    std::snprintf(line, sizeof(line), "\nPOLYGONS %lld %lld\n", (long long)nl2, (long long)nl2 * (vpf + 1));
    put(line);
    std::vector<int32_t> polys;
    polys.reserve((size_t)nl2 * (vpf + 1));
    for (int64_t f : leaves) {
      polys.push_back(vpf);
      for (int k = 0; k < vpf; ++k) polys.push_back(conn[(size_t)f * vpf + k]);
    }
    writeBigEndian(F.f, polys.data(), polys.size(), path);
    std::snprintf(line, sizeof(line), "\nPOINT_DATA %lld\nSCALARS relVort double 1\nLOOKUP_TABLE default\n",
                  (long long)nv);
    put(line);
    writeBigEndian(F.f, vz.data(), vz.size(), path);
    put("\nVECTORS velocity double\n");
    writeBigEndian(F.f, vv.data(), vv.size(), path);
    std::vector<double> cz, cv, ca;
    for (int64_t f : leaves) {
      cz.push_back(fz[f]);
      ca.push_back(fa[f]);
      for (int c = 0; c < 3; ++c) cv.push_back(fv[3 * f + c]);
    }
    std::snprintf(line, sizeof(line), "\nCELL_DATA %lld\nSCALARS relVort double 1\nLOOKUP_TABLE default\n",
                  (long long)nl2);
    put(line);
    writeBigEndian(F.f, cz.data(), cz.size(), path);
    put("\nSCALARS area double 1\nLOOKUP_TABLE default\n");
    writeBigEndian(F.f, ca.data(), ca.size(), path);
    put("\nVECTORS velocity double\n");
    writeBigEndian(F.f, cv.data(), cv.size(), path);
    put("\n");
  } catch (const Error& e) {
    return fail_code(e, nullptr);
  } catch (const std::exception& e) {
    return fail_code(fromStd(e), nullptr);
  }
  return LPM_OK;
}

}  // extern "C"
