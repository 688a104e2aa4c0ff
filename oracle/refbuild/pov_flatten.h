// pov_flatten.h -- the reference side of the drop-in boundary: a parsed
// SceneData flattened into the C ABI's PovGpuSceneDesc (include/povgpu.h),
// compiled against the reference's own headers.  This is the walk that
// View::StartRender would do once per view before creating the GPU render
// task (source/backend/scene/view.cpp:1141-1190); here it also feeds the
// scene-file dumps the tests compare with the project's scene generator.
#ifndef POV_FLATTEN_H
#define POV_FLATTEN_H

#include <cstdio>
#include <string>
#include <vector>

#include "povgpu.h"

namespace pov { class SceneData; }

namespace povgpu_ref {

// Owns every array the descriptor points at.
struct FlatScene
{
    std::vector<PovGpuObject>   objects;
    std::vector<PovGpuMaterial> materials;
    std::vector<PovGpuLight>    lights;
    std::vector<PovGpuMedia>    medias;
    std::vector<PovGpuPattern>  patterns;
    std::vector<PovGpuNormal>   normals;
    std::vector<PovGpuInterior> interiors;
    std::vector<int32_t>        object_interior;
    std::vector<PovGpuMesh>     meshes;
    std::vector<std::vector<float>>   mesh_vertices, mesh_normals;
    std::vector<std::vector<int32_t>> mesh_faces, mesh_normal_indices;
    PovGpuSceneDesc desc;
};

// Walks sd (after parsing and Build_Bounding_Slabs) into `out`: objects of
// SceneData::objects in order, light sources skipped, CSG children
// depth-first right after their parent -- the object ids the reference's
// Intersection::Object maps to.  Returns false and sets `why` (naming the
// object index) for what the GPU path does not take, as
// pov_gpu_scene_create would reject it.
bool FlattenScene(const pov::SceneData& sd, FlatScene& out, std::string& why);

// The scene file: the descriptor and its arrays as plain little-endian
// records (format in povray_gb300/scenefile.py).
bool WriteSceneFile(const FlatScene& f, const char* path);

}  // namespace povgpu_ref

#endif
