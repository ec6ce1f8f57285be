/*
 * gbsfm.h - C ABI of the engine-side scans around the bundle adjustment.
 *
 * The incremental engine runs three per-element loops over state it already
 * holds between BA calls; here each is one batched call:
 *   - gbsfm_triangulate_pair: triangulate2View_Vector
 *       (libs/sfm/include/mvg/sfm/sfm_robust.h:152-195), the per-match DLT
 *       and mean reprojection residual, with the keep decision its callers
 *       apply: Resection (libs/sfm/src/sfm_incremental_engine.cpp:977-1029:
 *       residual below each camera's threshold, positive depths, ray angle
 *       above 2 degrees) and MakeInitialPair3D (:492-533: robust-fit inlier,
 *       positive depths, ray angle);
 *   - gbsfm_reject_tracks: IncrementalReconstructionEngine::badTrackRejector
 *       (:1047-1140);
 *   - gbsfm_residual_histogram: IncrementalReconstructionEngine::
 *       ComputeResidualsHistogram (:1550-1616).
 * Cameras are the engine's BrownPinholeCamera
 * (libs/camera/include/mvg/camera/brown_pinhole_camera.h:44-140): rotation,
 * translation, focal length, principal point and radial K3 distortion, with
 * P = K [R | t].  Tracks are CSR over the cameras with one 3D point per track;
 * the observations of a track may come in any order (the reference's first
 * observation, which starts the ray-angle test, is the one of the lowest
 * camera index).  All computations are FP64.
 */
#ifndef GBSFM_H_
#define GBSFM_H_

#include <stdint.h>
#include "gbba.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gbsfm_camera {
  double R[9];                     /* rotation_matrix_, row-major */
  double t[3];                     /* translation_vector_ */
  double f, ppx, ppy, k1, k2, k3;  /* _f, _ppx, _ppy, _k1, _k2, _k3 */
} gbsfm_camera;

/* Pair triangulation with its keep filter.  cam1 / cam2 are host pointers;
 * x1, x2 [n][2] pixels; inlier [n] (NULL: every match) ; outputs X [n][3]
 * (TriangulateDLT, Euclidean), residual [n] (mean of the two PinholeCamera
 * residuals through P), keep [n] (1: the point enters the reconstruction),
 * num_kept (host, may be NULL).  keep = inlier && BrownPinholeCamera
 * residuals < max_residual1 / max_residual2 (pass +inf to skip the test, as
 * MakeInitialPair3D does) && both depths > 0 && AngleBetweenRay >
 * min_angle_deg.  Any output array may be NULL. */
gbba_status gbsfm_triangulate_pair(gbba_handle* handle, const gbsfm_camera* cam1, const gbsfm_camera* cam2,
                                   int64_t num_matches, const double* x1, const double* x2, const uint8_t* inlier,
                                   double max_residual1, double max_residual2, double min_angle_deg,
                                   double* X, double* residual, uint8_t* keep, int64_t* num_kept,
                                   int32_t memory);

/* Bad-track rejection.  cameras [num_cameras], points [num_tracks][3],
 * track_offsets [num_tracks+1], camera_index / xy per observation.  A
 * measurement is erased when its BrownPinholeCamera residual exceeds
 * `precision`; every measurement of a track is erased when the largest angle
 * between its first ray and any other is below min_track_angle_deg (3 in the
 * reference); a track that lost a measurement and keeps fewer than two is
 * removed.  Outputs obs_keep [N_o], track_keep [num_tracks] (either may be
 * NULL) and, on the host, the counts of erased measurements and removed
 * tracks (the reference returns their sum). */
gbba_status gbsfm_reject_tracks(gbba_handle* handle, const gbsfm_camera* cameras, int64_t num_cameras,
                                const double* points, int64_t num_tracks, const int64_t* track_offsets,
                                const uint32_t* camera_index, const double* xy, double precision,
                                double min_track_angle_deg, uint8_t* obs_keep, uint8_t* track_keep,
                                int64_t* rejected_measurements, int64_t* rejected_tracks, int32_t memory);

/* Residual statistics of every measurement: the BrownPinholeCamera residuals
 * rounded to float (as the reference stores them), their minimum, maximum,
 * mean and median (MinMaxMeanMedian, numeric.h:412-425) and the 10-bin
 * Histogram<double>(min, max, 10) of them (utils/histogram.h).  Filled only
 * when count > 1 (the reference returns -1 otherwise). */
typedef struct gbsfm_residual_stats {
  int64_t count;
  double min, max, mean, median;
  int64_t hist[10];
  int64_t underflow, overflow;
} gbsfm_residual_stats;

gbba_status gbsfm_residual_histogram(gbba_handle* handle, const gbsfm_camera* cameras, int64_t num_cameras,
                                     const double* points, int64_t num_tracks, const int64_t* track_offsets,
                                     const uint32_t* camera_index, const double* xy, gbsfm_residual_stats* stats,
                                     int32_t memory);

#ifdef __cplusplus
}
#endif
#endif /* GBSFM_H_ */
