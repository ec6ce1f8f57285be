/*
 * gbtri.h - C ABI of the GB300 batched triangulation kernels.
 *
 * Replaces the per-call Eigen JacobiSVD triangulation of the reference:
 *   - TriangulateDLT(P1, x1, P2, x2, Vec4* / Vec3*)
 *       libs/multiview/include/mvg/multiview/triangulation.h:12-20,
 *       libs/multiview/src/triangulation.cpp:10-29 (4x4 design, nullspace by
 *       SVD, libs/base/include/mvg/math/numeric.h:228-240);
 *   - TriangulateNView(x, Ps, Vec4*) and TriangulateNViewAlgebraic
 *       libs/multiview/include/mvg/multiview/triangulation_nview.h:12-15,
 *       libs/multiview/src/triangulation_nview.cpp:8-46;
 *   - Triangulation::compute(iter) / error(X) (iterated weighted linear
 *       method), libs/multiview/src/triangulation_nview.cpp:48-121, used by
 *       the global engine's per-track loop (sfm_global_engine.cpp:597-651).
 * The reference calls these once per track; here one call triangulates a
 * whole batch of tracks given as CSR (track_offsets) over a camera table.
 *
 * Projection matrices are row-major 3x4 (P = K[R|t]).  Homogeneous outputs
 * are unit vectors; like the reference's SVD nullspace their overall sign is
 * not specified.
 */
#ifndef GBTRI_H_
#define GBTRI_H_

#include <stdint.h>
#include "gbba.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gbtri_method {
  GBTRI_NVIEW = 0,            /* TriangulateNView: nullspace of the 3n x (4+n) design */
  GBTRI_NVIEW_ALGEBRAIC = 1,  /* TriangulateNViewAlgebraic: nullspace of the 2n x 4 design */
  GBTRI_ITERATIVE = 2         /* Triangulation::compute(3): Euclidean output + error() */
} gbtri_method;

/* Per-track status of the FP32 path. */
typedef enum gbtri_track_status {
  GBTRI_TRACK_OK = 0,
  GBTRI_TRACK_DEGENERATE = 1,    /* fewer than 2 views, a point at infinity or singular equations */
  GBTRI_TRACK_BEHIND_CAMERA = 2  /* min depth over the track's views <= 0 */
} gbtri_track_status;

/* Batched two-view DLT in FP64 (TriangulateDLT).  P1/P2 are [n][3][4] when
 * p_stride == 12, or a single shared 3x4 matrix each when p_stride == 0
 * (the triangulate2View_Vector case, sfm_robust.h:152-195).  x1/x2 are
 * [n][2].  Either output may be NULL: X_homogeneous [n][4] (unit vector),
 * X_euclidean [n][3]. */
gbba_status gbtri_dlt2_batched(gbba_handle* handle, int64_t n,
                               const double* P1, const double* P2, int64_t p_stride,
                               const double* x1, const double* x2,
                               double* X_homogeneous, double* X_euclidean,
                               int32_t memory);

/* Batched N-view triangulation in FP64.  track_offsets [num_tracks+1],
 * camera_index [N_o] into P [num_cameras][3][4], xy [N_o][2].
 * X: [num_tracks][4] (unit homogeneous) for GBTRI_NVIEW / _ALGEBRAIC,
 *    [num_tracks][3] for GBTRI_ITERATIVE.
 * error: GBTRI_ITERATIVE only, Triangulation::error(X) per track (sum of
 *    reprojection distances), or NULL.  Tracks may have any length: the
 *    nullspace is found from a per-track 4x4 reduction of the design, with
 *    O(1) state per track, instead of an SVD of the (3n) x (4+n) matrix. */
gbba_status gbtri_nview_batched(gbba_handle* handle, int32_t method,
                                const double* P, int64_t num_cameras,
                                const int64_t* track_offsets, const uint32_t* camera_index,
                                const double* xy, int64_t num_tracks,
                                double* X, double* error, int32_t memory);

/* The production path in FP32: the same estimators as gbtri_nview_batched
 * (`method`: GBTRI_NVIEW, the reference's TriangulateNView dehomogenised;
 * GBTRI_NVIEW_ALGEBRAIC; GBTRI_ITERATIVE, Triangulation::compute(3)) followed
 * by `gn_steps` Gauss-Newton steps on the reprojection error.
 * track_offsets are uint32 [num_tracks+1]; outputs X [num_tracks][3]
 * (Euclidean), status [num_tracks] (gbtri_track_status, may be NULL),
 * min_depth [num_tracks] (may be NULL). */
gbba_status gbtri_nview_batched_f32(gbba_handle* handle, int32_t method,
                                    const float* P, int64_t num_cameras,
                                    const uint32_t* track_offsets, const uint32_t* camera_index,
                                    const float* xy, int64_t num_tracks, int32_t gn_steps,
                                    float* X, uint8_t* status, float* min_depth,
                                    int32_t memory);

/* Gauss-Newton refinement of existing Euclidean points in FP64 (reprojection
 * error, `steps` iterations): X [num_tracks][3] in/out. */
gbba_status gbtri_refine_gn(gbba_handle* handle, const double* P, int64_t num_cameras,
                            const int64_t* track_offsets, const uint32_t* camera_index,
                            const double* xy, int64_t num_tracks, int32_t steps,
                            double* X, int32_t memory);

#ifdef __cplusplus
}
#endif
#endif /* GBTRI_H_ */
