// raytracer_overlap_direct_estimation -- drop-in for the reference's
// `raytracer_overlap_direct_estimation` (query/src/applications/raytracer_overlap_direct_estimation_main.cpp);
// the estimated overlap executable with the direct-estimation flags enabled.
#define RS_DIRECT 1
#include "raytracer_overlap_estimated.cpp"
