// Scene mesh of libclsph/scene.h:7-15. load() reads "scenes/<filename>" (a
// Wavefront OBJ; polygons become triangle fans) and computes one unit normal
// per face. Same arrays and the same multi-shape behaviour as the reference.
#ifndef _SCENE_H_
#define _SCENE_H_

#include <string>
#include <vector>

class scene {
 public:
  bool load(std::string filename);

  unsigned int face_count = 0;
  std::vector<float> face_normals;
  std::vector<float> vertices;
  std::vector<unsigned int> indices;
  // false (default): the reference's behaviour for files with several shapes
  // (the mesh is the last shape's; face_normals holds every shape's normals).
  // true: all shapes are concatenated into one mesh.
  bool fix_multi_shape = false;
};

#endif
