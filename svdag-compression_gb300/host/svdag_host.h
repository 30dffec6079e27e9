// Host-side helpers of the SVDAG build: seeded synthetic scenes and the OBJ
// writer.  These are not part of the GPU boundary (include/svdag_gpu.h); they
// feed it.
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

uint64_t svdag_synth_icosphere_count(uint32_t subdiv);
int svdag_synth_icosphere(uint32_t subdiv, double radius, double amp, uint64_t seed, float* out_tris);
uint64_t svdag_synth_terrain_count(uint32_t grid);
int svdag_synth_terrain(uint32_t grid, uint32_t octaves, double height, uint64_t seed, float* out_tris);
int svdag_synth_boxes(const float* lo, const float* hi, uint64_t n_boxes, float* out_tris);
int svdag_write_obj(const char* path, const float* tris, uint64_t n_tris, int pin_unit_cube);

/* OBJ scene loading (Scene::loadObj, src/symvox/scene.cpp:51-250) on
 * `threads` host threads (0: all cores), with the .bincache read / write of
 * the reference.  The triangles (9 floats each, Scene::getTrianglePtr
 * layout) stay owned by the scene. */
typedef struct svdag_scene svdag_scene;
int svdag_scene_load_obj(const char* path, uint32_t threads, int use_bincache, int write_bincache,
                         svdag_scene** out);
uint64_t svdag_scene_triangle_count(const svdag_scene* s);
const float* svdag_scene_triangles(const svdag_scene* s);
int svdag_scene_bbox(const svdag_scene* s, float bbox[6]);
void svdag_scene_free(svdag_scene* s);

#ifdef __cplusplus
}
#endif
