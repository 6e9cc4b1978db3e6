/*
 * lidar_gb300.h — C ABI of the GB300 (sm_103a) LiDAR perception library.
 *
 * Every entry point is `extern "C"`, takes plain pointers and sizes, returns an lp_status and
 * never throws. Host buffers are owned by the caller. Device buffers are owned by the context;
 * a context is not thread-safe (one per host thread), mirroring the reference's stateful,
 * single-threaded algorithm objects.
 *
 * Reference interfaces replaced (paths are inside YevgeniyEngineer/LiDAR-Processing-V2):
 *   lp_add_ring_info        Dataloader::addRingInfo               src/dataloader/src/dataloader.cpp:68-137
 *   lp_segment              Segmenter::segment<PointT>            lidar_processing_lib/src/segmenter.cpp:87-101
 *                           (+ Segmenter::image(), segmenter.hpp:163-166, as image_bgr_out)
 *   lp_noise_remove         NoiseRemover::filter                  lidar_processing_lib/src/noise_remover.cpp:38-68
 *   lp_cluster              Clusterer::cluster<PointT>            lidar_processing_lib/src/clusterer.cpp:43-53
 *   lp_convex_hull          Polygonizer::convexHull<PointXY>      lidar_processing_lib/src/polygonizer.cpp:33-91
 *   lp_antipodal_pairs      Polygonizer::findAntipodalPairsOfConvexHull  polygonizer.cpp:93-163
 *   lp_bounding_box_rotating_calipers  Polygonizer::boundingBoxRotatingCalipers  polygonizer.cpp:165-278
 *   lp_bounding_box_pca     Polygonizer::boundingBoxPrincipalComponentAnalysis  polygonizer.cpp:280-362
 *   lp_process_scan / lp_process_batch
 *                           Processor::run (segment → obstacle split → cluster → per-cluster
 *                           gather → convexHull), src/processor/src/processor.cpp:492-671
 *   lp_split_clouds         Processor::run's ground / obstacle / unsegmented clouds,
 *                           src/processor/src/processor.cpp:558-579
 *   lp_unpack_pointcloud2   convert<PointT>(PointCloud2 -> pcl cloud), src/processor/src/processor.cpp:42-179
 */
#ifndef LIDAR_GB300_H
#define LIDAR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t lp_status;

enum
{
    LP_OK = 0,
    LP_ERR_BAD_ARG = 1,   /* null pointer, zero capacity, malformed config */
    LP_ERR_CAPACITY = 2,  /* a fixed capacity was exceeded (e.g. the 200,000-voxel map) */
    LP_ERR_TIMEOUT = 3,   /* a bounded device-side wait ran out */
    LP_ERR_CUDA = 4,      /* a CUDA runtime call failed; see lp_last_error */
    LP_ERR_NO_DEVICE = 5, /* no CUDA device / library built without one */
    LP_ERR_INTERNAL = 6   /* device-side consistency check failed (error word set) */
};

/* Segmentation labels, segmenter.hpp:69-74. */
enum
{
    LP_LABEL_UNKNOWN = 0,
    LP_LABEL_GROUND = 1,
    LP_LABEL_OBSTACLE = 2
};

/* Noise labels, noise_remover.hpp:35-39. */
enum
{
    LP_NOISE_VALID = 0,
    LP_NOISE_NOISE = 1
};

#define LP_INVALID_CLUSTER (-1)

/* Mirrors SegmenterConfiguration, segmenter.hpp:87-112 (bools widened to int32). */
typedef struct lp_segmenter_config
{
    float elevation_up_deg;
    float elevation_down_deg;
    int32_t image_width;
    int32_t image_height;
    int32_t assume_unorganized_cloud;
    float grid_radial_spacing_m;
    float grid_slice_resolution_deg;
    float ground_height_threshold_m;
    float road_maximum_slope_m_per_m;
    float min_distance_m;
    float max_distance_m;
    float sensor_height_m;
    float kernel_threshold_distance_m;
    float amplification_factor;
    float z_min_m;
    float z_max_m;
} lp_segmenter_config;

/* Mirrors NoiseRemoverConfiguration, noise_remover.hpp:41-54. */
typedef struct lp_noise_remover_config
{
    float radius_multiplier_m_per_m;
    float min_search_radius_m;
    uint32_t min_neighbours;
} lp_noise_remover_config;

/* Mirrors ClustererConfiguration, clusterer.hpp:61-68. */
typedef struct lp_clusterer_config
{
    float voxel_grid_range_resolution_m;
    float voxel_grid_azimuth_resolution_deg;
    float voxel_grid_elevation_resolution_deg;
    uint32_t min_cluster_size;
} lp_clusterer_config;

/* Mirrors BoundingBox, polygonizer.hpp:75-81: corners[k] = {x, y}. */
typedef struct lp_bounding_box
{
    double corners[4][2];
    float area;
    float angle_rad;
    int32_t is_valid;
} lp_bounding_box;

/* Defaults equal to the reference structs' member initialisers. */
void lp_segmenter_config_default(lp_segmenter_config* cfg);
void lp_noise_remover_config_default(lp_noise_remover_config* cfg);
void lp_clusterer_config_default(lp_clusterer_config* cfg);

/* ------------------------------------------------------------------------------------------ */
/* Context                                                                                     */
/* ------------------------------------------------------------------------------------------ */
typedef struct lp_context lp_context;

lp_status lp_context_create(int32_t device, lp_context** out);
void lp_context_destroy(lp_context* ctx);
const char* lp_status_string(lp_status status);
/* Text of the last failure on this context ("" if none). */
const char* lp_last_error(const lp_context* ctx);
/* Number of kernels this context launched since creation (instrumentation). */
uint64_t lp_kernel_launch_count(const lp_context* ctx);

/* ------------------------------------------------------------------------------------------ */
/* Single-scan entry points (the reference's per-call form). Inputs and outputs in host memory. */
/* ------------------------------------------------------------------------------------------ */

/* Ring index per point from azimuth-quadrant transitions in input order; the first ring is
 * `first_ring` (63 in the reference) and each FOURTH->FIRST quadrant change decrements it down
 * to 0. xyzi: n x 4 floats. */
lp_status lp_add_ring_info(lp_context* ctx, const float* xyzi, uint32_t n, uint16_t first_ring,
                           uint16_t* ring_out);

/* A field the cloud does not carry (lp_unpack_pointcloud2). */
#define LP_NO_FIELD 0xffffffffu

/* Unpacks a sensor_msgs/PointCloud2 byte buffer as convert<PointT> does (processor.cpp:42-179):
 * point (row, col) starts at row * row_step + col * point_step; offsets[5] are the byte offsets of
 * x, y, z, intensity (float32) and ring (uint16) within a point, intensity and ring LP_NO_FIELD when
 * absent (intensity then 0). Little-endian data, fields need not be aligned. data: height *
 * row_step bytes; xyzi_out: width * height x 4 floats; ring_out: NULL or width * height uint16. */
lp_status lp_unpack_pointcloud2(lp_context* ctx, const uint8_t* data, uint32_t width, uint32_t height,
                                uint32_t point_step, uint32_t row_step, const uint32_t* offsets, float* xyzi_out,
                                uint16_t* ring_out);

/* A point of the processor's coloured clouds (pcl::PointXYZRGB's position and colour; a = 255). */
typedef struct lp_xyzrgb
{
    float x, y, z;
    uint8_t r, g, b, a;
} lp_xyzrgb;

/* The processor's three clouds from a segmentation (processor.cpp:558-579): the points labelled
 * GROUND coloured (124, 252, 0), OBSTACLE (200, 0, 0) and every other label (255, 255, 0), each in
 * input order. xyzi: n x 4 floats; labels: n uint32 (LP_LABEL_*). ground / obstacle / unsegmented:
 * host buffers of n entries each (any may be NULL: that cloud is counted, not copied). counts[3]
 * receives the three cloud sizes. */
lp_status lp_split_clouds(lp_context* ctx, const float* xyzi, const uint32_t* labels, uint32_t n, lp_xyzrgb* ground,
                          lp_xyzrgb* obstacle, lp_xyzrgb* unsegmented, uint32_t* counts);

/* The processor's per-cluster products after the hulls (processor.cpp:609-797), from one scan's
 * pipeline outputs: the clustered cloud, the vehicle gates and the boundary marker geometry.
 * - clustered cloud (processor.cpp:627-658): every clustered point, grouped by cluster label in
 *   label order, input order within a label, coloured per label with three std::rand() % 256
 *   draws (r, g, b). The reference never seeds rand(), so the draws continue glibc's default
 *   stream; rand_draws says how many the process made before this scan (0 after start-up; each
 *   scan with K clusters makes 3K).
 * - vehicle gates (processor.cpp:675-771; perform_polygon_simplification, false in the reference):
 *   a cluster of more than 150 points with a hull of at least 3 vertices, height (z range) and
 *   hull-area volume inside the vehicle table's limits (processor.hpp:60-192), is boxed by
 *   rotating calipers over ALL its points in input order (as the reference calls it), and
 *   classified by the first vehicle type whose length, width, height, volume and area bounds it
 *   meets when the hull fills more than 0.4 of the box.
 * - boundary markers (convertPolygonPointsToMarker, processor.cpp:241-343): LINE_LIST points of the
 *   polygon (the box corners for a classified cluster, else the hull) at z_min and z_max and the
 *   vertical edges, 6 per polygon vertex; none for a polygon of fewer than 3 points. */
typedef struct lp_object_config
{
    int32_t vehicle_gates; /* 1: evaluate the vehicle gates */
    uint32_t reserved;
    uint64_t rand_draws;   /* std::rand() calls made in the process before this scan */
} lp_object_config;

typedef struct lp_object_output
{
    lp_xyzrgb* clustered_cloud;  /* optional; capacity >= clustered points (labels >= 0) */
    int32_t* vehicle_class;      /* optional, n_clusters: vehicle type 0-4 (compact car, sedan, SUV,
                                    truck, minivan), -1 where the cluster is not boxed */
    lp_bounding_box* gate_boxes; /* optional, n_clusters: the gate's calipers box (invalid where the
                                    gate did not reach it) */
    uint32_t* marker_offsets;    /* optional, n_clusters + 1: first marker point of each cluster */
    double* marker_points;       /* optional, marker_capacity x 3 doubles (x, y, z) */
    uint32_t marker_capacity;
    /* Written by the library. */
    uint32_t n_clustered;
    uint32_t n_marker_points;
} lp_object_output;

/* xyzi: n x 4 floats; cluster_labels: n (LP_INVALID_CLUSTER for unclustered points); hull_offsets
 * (n_clusters + 1), hull_indices (local to each cluster), z_min, z_max (n_clusters): the outputs of
 * lp_process_scan for that cloud. All buffers are host memory. LP_ERR_CAPACITY when the marker
 * points exceed marker_capacity (n_marker_points then says how many are needed). */
lp_status lp_cluster_objects(lp_context* ctx, const float* xyzi, const int32_t* cluster_labels, uint32_t n,
                             uint32_t n_clusters, const uint32_t* hull_offsets, const int32_t* hull_indices,
                             const float* z_min, const float* z_max, const lp_object_config* cfg,
                             lp_object_output* out);

/* Ground segmentation. xyzi: n x 4 floats (x, y, z, intensity). ring: per-point ring index, or
 * NULL for a cloud without a ring field (the height index then comes from the elevation angle,
 * as for pcl::PointXYZ/XYZI). labels_out: n uint32 (LP_LABEL_*). image_bgr_out: optional
 * image_height x image_width x 3 bytes, the jump-convolution colour image. */
lp_status lp_segment(lp_context* ctx, const float* xyzi, const uint16_t* ring, uint32_t n,
                     const lp_segmenter_config* cfg, uint32_t* labels_out, uint8_t* image_bgr_out);

/* Dynamic-radius outlier removal. xyz: n points, `stride` floats apart (3 for
 * std::array<float,3>, 4 for XYZI). labels_out: n bytes (LP_NOISE_*). */
lp_status lp_noise_remove(lp_context* ctx, const float* xyz, uint32_t stride, uint32_t n,
                          const lp_noise_remover_config* cfg, uint8_t* labels_out);

/* Curved-voxel clustering. labels_out: n int32, cluster id or LP_INVALID_CLUSTER. */
lp_status lp_cluster(lp_context* ctx, const float* xyz, uint32_t stride, uint32_t n,
                     const lp_clusterer_config* cfg, int32_t* labels_out);

/* Convex hull (Andrew's monotone chain). xy: n x 2 doubles. indices_out: capacity >= n + 1;
 * *n_out receives the hull size. Counter-clockwise, starting at the lexicographic minimum. */
lp_status lp_convex_hull(lp_context* ctx, const double* xy, uint32_t n, int32_t* indices_out,
                         uint32_t* n_out);

/* Convex hull without any device allocation. This entry point has no counterpart in the
 * reference library. It is for callers that cannot call cudaMalloc: real-time loops that reserve
 * all memory up front (an allocation can synchronise the device and stall other work), plugin
 * hosts whose allocation policy forbids it, and paths where an allocation failure cannot be
 * handled. Inputs and outputs are DEVICE buffers owned by the caller: d_xy holds n x 2 doubles,
 * d_indices_out at least n + 1 int32, d_n_out one uint32 (the hull size). Results equal
 * lp_convex_hull's. The kernel's working memory is a static device array of 2.1 MiB that every
 * GPU which loads the library keeps until the process exits; n above LP_NOALLOC_HULL_MAX_POINTS
 * is rejected with LP_ERR_CAPACITY before anything runs. The first call on a device looks up that
 * array's device address (once per device, with the device current), so make that first call
 * before any stream capture. That address is kept for the life of the process: after a
 * cudaDeviceReset (or any teardown of the device's primary context) the library reloads and the
 * kept address is stale, so this entry point must not be called on that device again. The work
 * is enqueued on `stream` (a cudaStream_t, NULL for the default stream) and the call returns
 * without waiting; the status reports this call's own launch (LP_ERR_CUDA if it was refused).
 * All calls share the one array: calls whose kernels overlap on the GPU (other threads, other
 * streams) race and must be serialised by the caller. */
#define LP_NOALLOC_HULL_MAX_POINTS 65536u
lp_status lp_convex_hull_noalloc(const double* d_xy, uint32_t n, int32_t* d_indices_out, uint32_t* d_n_out,
                                 void* stream);

/* Antipodal pairs of a convex polygon (Shamos). pairs_out: capacity pairs x 2 int32. */
lp_status lp_antipodal_pairs(lp_context* ctx, const double* hull_xy, uint32_t n,
                             int32_t* pairs_out, uint32_t capacity, uint32_t* n_pairs);

lp_status lp_bounding_box_rotating_calipers(lp_context* ctx, const double* hull_xy, uint32_t n,
                                            lp_bounding_box* out);
lp_status lp_bounding_box_pca(lp_context* ctx, const double* hull_xy, uint32_t n,
                              lp_bounding_box* out);

/* ------------------------------------------------------------------------------------------ */
/* Whole per-scan pipeline, one scan or a batch of scans in one launch sequence.              */
/* ------------------------------------------------------------------------------------------ */
typedef struct lp_pipeline_config
{
    lp_clusterer_config cluster;
    lp_noise_remover_config noise;
    int32_t enable_noise_removal; /* 1: DROR on the input cloud, segment the VALID points */
    int32_t compute_ring;         /* 1: derive ring indices on the device (lp_add_ring_info) */
    uint16_t first_ring;          /* start ring for compute_ring (63 in the reference) */
    uint16_t reserved0;
    int32_t compute_obb;          /* 1: rotating-calipers and PCA boxes per cluster */
} lp_pipeline_config;

void lp_pipeline_config_default(lp_pipeline_config* cfg);

typedef struct lp_scan_input
{
    const float* xyzi;    /* n x 4 floats */
    const uint16_t* ring; /* n ring indices, or NULL (compute_ring, or unorganized cloud) */
    uint32_t n;
    lp_segmenter_config seg;
} lp_scan_input;

typedef struct lp_scan_output
{
    /* Per input point (n entries each). */
    uint8_t* noise_labels;   /* optional; LP_NOISE_* (VALID everywhere when DROR is off) */
    uint32_t* seg_labels;    /* optional; LP_LABEL_* (UNKNOWN for points removed as noise) */
    int32_t* cluster_labels; /* optional; cluster id of obstacle points, else LP_INVALID_CLUSTER */
    /* Per cluster. Hull indices are local to the cluster: they index the cluster's points in
     * input order, exactly as the reference's per-cluster gather + convexHull produce them. */
    uint32_t cluster_capacity;
    uint32_t hull_capacity;
    uint32_t* hull_offsets;       /* cluster_capacity + 1 */
    int32_t* hull_indices;        /* hull_capacity */
    float* z_min;                 /* optional, cluster_capacity */
    float* z_max;                 /* optional, cluster_capacity */
    lp_bounding_box* obb_calipers; /* optional, cluster_capacity */
    lp_bounding_box* obb_pca;      /* optional, cluster_capacity */
    /* Written by the library. */
    uint32_t n_obstacles;
    uint32_t n_clusters;
    uint32_t n_hull_indices;
    lp_status status;
} lp_scan_output;

lp_status lp_process_scan(lp_context* ctx, const lp_pipeline_config* cfg, const lp_scan_input* scan,
                          lp_scan_output* out);
lp_status lp_process_batch(lp_context* ctx, const lp_pipeline_config* cfg,
                           const lp_scan_input* scans, lp_scan_output* outs, uint32_t nscans);

#ifdef __cplusplus
}
#endif

#endif /* LIDAR_GB300_H */
