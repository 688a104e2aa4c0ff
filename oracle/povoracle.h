/*
 * povoracle.h -- CPU restatement of the reference trace path.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is the checker for libpovgpu: only
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load
 * it.  It consumes the same PovGpuSceneDesc as the GPU library and follows
 * the reference's FP64 algorithm (file:line citations in povoracle.c).
 * It is pinned against golden vectors produced by the reference itself
 * (oracle/refbuild/pov_oracle.cpp, fixtures under tests/golden/).
 */
#ifndef POVORACLE_H
#define POVORACLE_H

#include "../include/povgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct PovOracle PovOracle;

int  pov_oracle_create(const PovGpuSceneDesc* desc, PovOracle** out, int32_t* bad_index);
void pov_oracle_destroy(PovOracle* o);
void pov_oracle_tree_info(const PovOracle* o, int32_t* top_nodes, int32_t* mesh_nodes);
/* Entry i of the pattern random table (the cells pattern's values). */
double pov_oracle_pattern_rand(int32_t i);

/* Trace::FindIntersection for each ray (origins/directions: 3 doubles each). */
int  pov_oracle_trace_rays(PovOracle* o, const double* origins, const double* directions,
                           int32_t n, PovGpuHit* hits);

/* Renders the pixel rectangle [x0,x1) x [y0,y1) (row-major RGBT floats)
 * with `threads` worker threads (0 = one per online CPU).  stats may be
 * NULL. */
int  pov_oracle_render(PovOracle* o, const PovGpuRenderParams* params, int32_t x0, int32_t y0,
                       int32_t x1, int32_t y1, int32_t threads, float* out_rgbt, PovGpuStats* stats);

/* Radiosity renders need the reference's pretrace jitter table
 * (RadiosityTask's RandomDoubleSequence, tests/golden/pretrace_jitter.npy);
 * the table is borrowed, not copied. */
int  pov_oracle_set_pretrace_jitter(PovOracle* o, const double* table, int32_t n);

/* Converged radiosity, the FP64 ground truth of radiosity images (no
 * counterpart in the reference): the final trace of the given pixels
 * (x, y pairs of the full image; row-major RGBT floats out, one per pixel)
 * with every radiosity query answered without the sample cache, by
 * counts[d] stratified cosine-weighted sample rays at bounce depth d
 * (counts shorter than the recursion depth repeat their last entry),
 * summed in FP64.  `seed` fixes the per-pixel random sequences; the result
 * does not depend on `threads`. */
int  pov_oracle_render_converged(PovOracle* o, const PovGpuRenderParams* params, const int32_t* pixels,
                                 int32_t n, const int32_t* counts, int32_t ncounts, uint64_t seed,
                                 int32_t threads, float* out_rgbt, PovGpuStats* stats);

/* Per-ray work counters of the restated traversal, for the roofline byte
 * model: node boxes tested and primitives tested over the given rays. */
int  pov_oracle_count_work(PovOracle* o, const double* origins, const double* directions,
                           int32_t n, uint64_t* boxes_tested, uint64_t* prims_tested);

#ifdef __cplusplus
}
#endif
#endif
