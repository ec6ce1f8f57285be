/*
 * gbsfm.h - C ABI of the engine-side work around the bundle adjustment.
 *
 * The incremental engine runs per-element loops over state it already holds
 * between BA calls; here each is one batched call:
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
 *       ComputeResidualsHistogram (:1550-1616);
 *   - gbsfm_pack_ba / gbsfm_unpack_ba: BundleAdjustment's problem assembly
 *       and write-back (:1250-1393, 1475-1546);
 *   - gbsfm_acransac_score: the hypothesis scoring of robustResection's
 *       AC-RANSAC (libs/sfm/include/mvg/sfm/sfm_robust.h:207-254).
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

/* ---- Problem assembly ----------------------------------------------------
 * IncrementalReconstructionEngine::BundleAdjustment packs its std::map state
 * into a BA_Problem_data_camMotionAndIntrinsic<6,6>
 * (libs/sfm/src/sfm_incremental_engine.cpp:1250-1393) and writes the refined
 * parameters back after the solve (:1475-1546).  Here the engine state is a
 * set of dense arrays, the pack is one pass over the track entries and the
 * write-back one pass over the cameras, so the state can stay in device
 * memory between BA calls.
 *
 * Engine state, every map in its key order:
 *   map_Camera           -> cameras[image] where reconstructed[image] != 0
 *   map_images_id_per_intrinsic_group_ -> intrinsic_group[image] (the
 *                           ordinal of the image's group among the keys)
 *   map_intrinsics_per_group_ -> group_intrinsics [G][6] f, ppx, ppy, k1, k2, k3
 *   map_features_        -> CSR feature_offsets [num_images+1] over
 *                           features [num_features][2] (ScalePointFeature x, y)
 *   map_3d_points        -> points [num_points][3], ascending track id
 *   map_reconstructed_   -> CSR track_offsets [num_points+1] over the entries
 *                           (track_image, track_feature), image id ascending
 *                           inside a track (SubmapTrack order). */
typedef struct gbsfm_engine_state {
  int64_t num_images;
  const gbsfm_camera* cameras;       /* [num_images] */
  const uint8_t* reconstructed;      /* [num_images] */
  const uint32_t* intrinsic_group;   /* [num_images] */
  int64_t num_intrinsic_groups;
  const double* group_intrinsics;    /* [num_intrinsic_groups][6] */
  int64_t num_features;
  const int64_t* feature_offsets;    /* [num_images+1] */
  const float* features;             /* [num_features][2] */
  int64_t num_points;
  const double* points;              /* [num_points][3] */
  int64_t num_entries;               /* track_offsets[num_points] */
  const int64_t* track_offsets;      /* [num_points+1] */
  const uint32_t* track_image;       /* [num_entries] */
  const uint32_t* track_feature;     /* [num_entries] */
} gbsfm_engine_state;

/* Which extrinsic block the pack holds constant.  The reference locks
 * mutable_camera_extrinsic_for_observation(ordinal of vec_added_order_[0])
 * (:1437-1443), an accessor that takes an observation index
 * (libs/sfm/include/mvg/sfm/problem_data_container.h:93-95): the block of
 * observation number `ordinal`.  GBSFM_LOCK_AS_REFERENCE reproduces that;
 * GBSFM_LOCK_FIRST_ADDED locks the first-added camera itself. */
typedef enum gbsfm_lock {
  GBSFM_LOCK_AS_REFERENCE = 0,
  GBSFM_LOCK_FIRST_ADDED = 1,
  GBSFM_LOCK_NONE = 2
} gbsfm_lock;

/* Outputs of the pack, sized for the worst case by the caller: extrinsics
 * [num_images][6], intrinsics [G][6], points [num_points][3], observations
 * [num_entries][2], the three index arrays [num_entries], camera_constant
 * and camera_image [num_images] (both may be NULL).  The layout is the
 * reference's parameters_ split in three: extrinsics (angle-axis from
 * ceres::RotationMatrixToAngleAxis, then t) in ascending image id,
 * intrinsic groups in key order, points in track order; observations keep
 * the track-major order, dropping entries of images without a camera.  It is
 * a gbba_problem of camera model GBBA_RADIAL_K3 as it stands. */
typedef struct gbsfm_ba_arrays {
  double* extrinsics;
  double* intrinsics;
  double* points;
  double* observations;
  uint32_t* camera_index;
  uint32_t* intrinsic_index;
  uint32_t* point_index;
  uint8_t* camera_constant;   /* 1 on the locked block */
  uint32_t* camera_image;     /* image id of each camera ordinal */
  int64_t num_cameras;        /* out */
  int64_t num_observations;   /* out: observations written */
  int64_t measurements;       /* out: sum of the track sizes, the reference's num_observations_ */
  int64_t locked_camera;      /* out: ordinal of the locked block, -1 for none */
} gbsfm_ba_arrays;

/* first_added_image: vec_added_order_[0], or -1 when the engine has added no
 * image.  Arrays of `state` and `out` are in `memory`.  Entries that name an
 * image or a feature outside the state, offsets that are not a CSR of
 * num_entries entries and intrinsic groups out of range return
 * GBBA_ERROR_INVALID_ARGUMENT (the reference indexes its maps unchecked). */
gbba_status gbsfm_pack_ba(gbba_handle* handle, const gbsfm_engine_state* state, int64_t first_added_image,
                          int32_t lock, gbsfm_ba_arrays* out, int32_t memory);

/* Write-back: for camera ordinal c, cameras[camera_image[c]] becomes the
 * BrownPinholeCamera of R = ceres::AngleAxisToRotationMatrix(extrinsics[c]),
 * t = extrinsics[c][3..5] and the intrinsics of its group
 * intrinsics[intrinsic_group[camera_image[c]]] (:1491-1516).  The points and
 * the groups' intrinsics go back as they are (:1481-1489, 1519-1529): the
 * packed arrays may be the engine's own. */
gbba_status gbsfm_unpack_ba(gbba_handle* handle, int64_t num_cameras, const double* extrinsics,
                            const uint32_t* camera_image, const double* intrinsics, int64_t num_intrinsic_groups,
                            const uint32_t* intrinsic_group, int64_t num_images, gbsfm_camera* cameras,
                            int32_t memory);

/* ---- AC-RANSAC hypothesis scoring ------------------------------------------
 * The per-model body of ACRANSAC's main loop
 * (libs/feature/include/mvg/feature/estimator_acransac.h:170-200) as used by
 * robustResection (libs/sfm/include/mvg/sfm/sfm_robust.h:207-254), for a
 * batch of candidate models: the squared reprojection error of every
 * correspondence (ResectionSquaredResidualError, sfm_robust.h:197-204:
 * |Project(P, X) - x|^2, P in the kernel's normalised image frame), sorted
 * ascending with ties in index order (std::sort of (error, index) pairs),
 * and bestNFA (estimator_acransac.h:75-97) over the sorted errors with the
 * float tables logcombi(k, n) and logcombi(sample_size, k) (:40-65).  Each
 * model's NFA, inlier count k and threshold e[k-1] come back; a model none
 * of whose errors passes max_threshold gets NFA +inf, k = sample_size and
 * threshold +inf (the reference leaves such a model unused).  The sampling
 * and the adaptive loop around it stay with the caller. */
typedef struct gbsfm_acransac_params {
  int32_t sample_size;   /* Kernel::MINIMUM_SAMPLES: 6 (six-point DLT) or 3 (P3P) */
  int32_t max_models;    /* Kernel::MAX_MODELS: 1 or 4; loge0 = log10(max_models (n - sample_size)) */
  double logalpha0;      /* log10(pi) for both resection kernels */
  double mult_error;     /* 1.0: point-to-point error */
  double max_threshold;  /* +inf, or precision * normalizer2(0,0)^2 */
} gbsfm_acransac_params;

/* x2d [num_points][2] (normalised, as the kernel adaptor holds them), x3d
 * [num_points][3], models [num_models][12] (row-major 3x4).  Outputs nfa,
 * num_inliers, error_max [num_models]; order [num_models][num_points] the
 * sorted correspondence indices (the inliers of model h are
 * order[h][0 .. num_inliers[h]-1]), or NULL.  num_points must exceed
 * sample_size (ACRANSAC returns early otherwise). */
gbba_status gbsfm_acransac_score(gbba_handle* handle, const gbsfm_acransac_params* params, int64_t num_points,
                                 const double* x2d, const double* x3d, int64_t num_models, const double* models,
                                 double* nfa, int32_t* num_inliers, double* error_max, uint32_t* order,
                                 int32_t memory);

#ifdef __cplusplus
}
#endif
#endif /* GBSFM_H_ */
