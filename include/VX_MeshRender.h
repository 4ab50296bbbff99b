// CVX_MeshRender: deformed surface mesh of a CVoxelyze (same public interface as the reference's
// include/VX_MeshRender.h:22-59).  The mesh topology (exposed faces, shared vertices, edges) is
// built on the host in the reference's order; updateMesh computes the vertex positions and quad
// normals on the GPU from the current state (vxg_mesh_update) and the quad colours on the host.
// glDraw needs an OpenGL context, which this library does not use: it draws nothing.  The buffers
// are readable directly (headless use) and saveObj writes them as a Wavefront OBJ file.
#ifndef VX_GB300_MESHRENDER_H
#define VX_GB300_MESHRENDER_H

#include <vector>

#include "Voxelyze.h"

class CVX_MeshRender {
 public:
  enum viewColoring { MATERIAL, FAILURE, STATE_INFO };

  CVX_MeshRender(CVoxelyze* voxelyzeInstance);
  void generateMesh();
  void updateMesh(viewColoring colorScheme = MATERIAL, CVoxelyze::stateInfoType stateType = CVoxelyze::DISPLACEMENT);
  void saveObj(const char* filePath);
  void glDraw();

  // headless access (extension of the reference API)
  const std::vector<float>& vertexPositions() const { return vertices; }  // x, y, z per vertex
  const std::vector<int>& quadVertices() const { return quads; }          // 4 vertex indices per quad
  const std::vector<float>& quadColorValues() const { return quadColors; }
  const std::vector<float>& quadNormalValues() const { return quadNormals; }
  const std::vector<int>& quadVoxels() const { return quadVoxIndices; }   // voxel of each quad
  const std::vector<int>& lineVertices() const { return lines; }          // 2 vertex indices per edge
  bool ok() const { return good; }  // false when the last update could not run on the GPU

 private:
  CVoxelyze* vx;
  std::vector<float> vertices;
  std::vector<int> vertexLinks;  // 8 voxel indices per vertex in voxelCorner order, -1 for none
  std::vector<int> quads;
  std::vector<float> quadColors;
  std::vector<int> quadVoxIndices;
  std::vector<float> quadNormals;
  std::vector<int> lines;
  bool uploaded = false;
  bool good = true;

  float jetMapR(float val) { if (val < 0.5f) return 0.0f; else if (val > 0.75f) return 1.0f; else return val * 4 - 2; }
  float jetMapG(float val) { if (val < 0.25f) return val * 4; else if (val > 0.75f) return 4 - val * 4; else return 1.0f; }
  float jetMapB(float val) { if (val > 0.5f) return 0.0f; else if (val < 0.25f) return 1.0f; else return 2 - val * 4; }
  float linkMaxColorValue(CVX_Voxel* pV, CVoxelyze::stateInfoType coloring);
};

#endif
