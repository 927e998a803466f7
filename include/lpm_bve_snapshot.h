/* lpm_bve_snapshot.h -- checkpoint / restart of a BVE state and legacy-VTK output.
 *
 * The reference writes its state through VTK (Polymesh2dVtkInterface, used by
 * tests/LpmBVETest.cpp:98-106 and :228-238) or netCDF (src/LpmNetCDF.hpp:23-103), both absent
 * here.  These entry points cover the same needs without those libraries:
 *   - a binary snapshot of every array of lpm_bve_state (positions, vorticity, velocity at
 *     vertices and faces, areas, mask) with the mesh seed/level, time, dt and Omega, restored bit
 *     for bit (a run stepped on from it builds a new plan from the restored positions, so it
 *     matches the uninterrupted run to the rounding of the summation order);
 *   - a legacy VTK PolyData file (vertices as points, leaf faces as polygons, relative vorticity
 *     and velocity as point and cell data, face area) that VTK readers and ParaView open.
 * Arrays may live on the device or the host.  Device and managed arrays are copied on `stream`,
 * host arrays with memcpy.  Every call synchronises `stream` when a CUDA device is present; with
 * host arrays the calls also work without one (stream NULL), e.g. for post-processing.
 * Errors return a negative status and print a message on stderr.
 */
#ifndef LPM_BVE_SNAPSHOT_H
#define LPM_BVE_SNAPSHOT_H

#include "lpm_bve.h"

#ifdef __cplusplus
extern "C" {
#endif

int lpm_bve_snapshot_write(const char* path, const lpm_bve_state* st, int seed, int level, double t, double dt,
                           double omega, lpm_stream_t stream);
/* Header only: sizes and metadata, so a caller can allocate the state before reading. */
int lpm_bve_snapshot_info(const char* path, int* seed, int* level, int64_t* nverts, int64_t* nfaces, double* t,
                          double* dt, double* omega);
/* Restores positions, vorticity and velocity into the caller's arrays.  The sizes must match and
 * the state's face areas and mask must equal the snapshot's (LPM_ERR_INVALID_ARGUMENT otherwise);
 * they are checked, not written. */
int lpm_bve_snapshot_read(const char* path, const lpm_bve_state* st, double* t, lpm_stream_t stream);
/* Legacy VTK PolyData of the state on mesh (seed, level). */
int lpm_bve_vtk_write(const char* path, const lpm_bve_state* st, int seed, int level, lpm_stream_t stream);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* LPM_BVE_SNAPSHOT_H */
