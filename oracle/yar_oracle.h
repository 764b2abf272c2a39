/*
 * yar_oracle.h - TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C CPU restatement of the reference renderer's hot path (kd-tree
 * traversal, watertight intersection, sampler, shading, BSDFs, delta
 * scattering, MIS direct lighting and the path loop of kennyalive/YAR
 * src/ref), used by tests/,
 * __graft_entry__.smoke() and the cpu_baseline leg of bench.py as the checker
 * of the CUDA path.  The product never links or calls it.
 *
 * Parity of this restatement is pinned against the reference itself
 * (oracle/_ref/yar_ref, built from the reference sources by
 * oracle/build_ref.sh) and against the golden vectors in tests/golden/.
 */
#ifndef YAR_ORACLE_H
#define YAR_ORACLE_H

#include "yar_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Per-ray traversal work, counted in the reference's visit order
 * (the algorithmic-bytes figure of the ray-cast roofline). */
typedef struct oracle_ray_stats {
    uint64_t nodes;          /* kd-nodes fetched (interior + leaf headers), both levels */
    uint64_t leaf_words;     /* primitive-index words read from leaves beyond word1 */
    uint64_t triangle_tests; /* watertight tests (after visibility filtering) */
    uint64_t object_visits;  /* scene-leaf object entries (ray transforms) */
} oracle_ray_stats;

/* KdTree::intersect over the scene tree (src/ref/kdtree.cpp:219-327). */
int oracle_cast_closest(const yar_flat_scene* scene, const yar_ray* rays, uint32_t n,
                        float* t, uint32_t* prim, uint32_t* object, float* bary,
                        oracle_ray_stats* stats);
/* KdTree::intersect_any over the scene tree (src/ref/kdtree.cpp:329-439). */
int oracle_cast_any(const yar_flat_scene* scene, const yar_ray* rays, uint32_t n,
                    uint8_t* occluded, oracle_ray_stats* stats);

/* intersect_triangle_watertight (src/ref/intersection.cpp:53-113); returns t or +inf. */
float oracle_intersect_triangle_watertight(const float origin[3], const float direction[3],
                                           const float p0[3], const float p1[3], const float p2[3],
                                           float barycentrics[3]);

/* pcg32 (third-party/pcg/pcg_basic.c:46-75) */
typedef struct oracle_pcg32 {
    uint64_t state;
    uint64_t inc;
} oracle_pcg32;
void oracle_pcg32_seed(oracle_pcg32* rng, uint64_t initstate, uint64_t initseq);
uint32_t oracle_pcg32_next(oracle_pcg32* rng);
float oracle_pcg32_float(oracle_pcg32* rng);

/* Stratified_Pixel_Sampler::next_pixel for one pixel (src/ref/pixel_sampling.cpp:54-141):
 * image[2*spp], s1d[spp*n1d], s2d[2*spp*n2d] in the reference's layout. */
void oracle_pixel_samples(uint32_t stream_id, int nx, int ny, int n1d, int n2d,
                          float* image, float* s1d, float* s2d);

/* render_scene (src/ref/reference_renderer.cpp:331-584) restricted to the
 * implemented path; rgb has render_region size. Returns YAR_OK or an error. */
int oracle_render(const yar_flat_scene* scene, float* rgb, double* variance,
                  int32_t row_begin, int32_t row_end, int32_t thread_count);

/* oracle_render with the sines and cosines of sampled angles either from the C
 * library (0, as the reference computes them) or correctly rounded (1, as the
 * CUDA path computes them).  The choice stays for later oracle_render calls. */
int oracle_render_trig(const yar_flat_scene* scene, float* rgb, double* variance,
                       int32_t row_begin, int32_t row_end, int32_t thread_count,
                       int32_t correctly_rounded_trig);

#ifdef __cplusplus
}
#endif
#endif
