// CVX_MeshRender for the drop-in API: mesh topology on the host in the reference's order
// (src/VX_MeshRender.cpp:49-138), vertex positions and quad normals on the GPU (vxg_mesh_update),
// quad colours on the host (src/VX_MeshRender.cpp:181-236), OBJ output (:238-252).
#include "VX_MeshRender.h"

#include <algorithm>
#include <cfloat>
#include <cstdint>
#include <fstream>
#include <unordered_map>

#include "vx_host.h"
#include "vxg.h"

namespace {

// the four corners of the exposed face in each link direction (X+, X-, Y+, Y-, Z+, Z-), in the
// order the quad lists its vertices; corner bits are x << 2 | y << 1 | z as in voxelCorner
const int kFaceCorners[6][4] = {
    {CVX_Voxel::PNN, CVX_Voxel::PPN, CVX_Voxel::PPP, CVX_Voxel::PNP},
    {CVX_Voxel::NNN, CVX_Voxel::NNP, CVX_Voxel::NPP, CVX_Voxel::NPN},
    {CVX_Voxel::NPN, CVX_Voxel::NPP, CVX_Voxel::PPP, CVX_Voxel::PPN},
    {CVX_Voxel::NNN, CVX_Voxel::PNN, CVX_Voxel::PNP, CVX_Voxel::NNP},
    {CVX_Voxel::NNP, CVX_Voxel::PNP, CVX_Voxel::PPP, CVX_Voxel::NPP},
    {CVX_Voxel::NNN, CVX_Voxel::NPN, CVX_Voxel::PPN, CVX_Voxel::PNN},
};

uint64_t grid_key(int x, int y, int z) {
  const uint64_t B = 1u << 20;
  return ((uint64_t)(x + B) << 42) | ((uint64_t)(y + B) << 21) | (uint64_t)(z + B);
}

}  // namespace

CVX_MeshRender::CVX_MeshRender(CVoxelyze* voxelyzeInstance) : vx(voxelyzeInstance) { generateMesh(); }

void CVX_MeshRender::generateMesh() {  // VX_MeshRender.cpp:49-138
  vertices.clear();
  vertexLinks.clear();
  quads.clear();
  quadColors.clear();
  quadVoxIndices.clear();
  quadNormals.clear();
  lines.clear();
  uploaded = false;

  struct GridVertex {
    int x, y, z, index;
  };
  std::unordered_map<uint64_t, int> vIndMap;  // lattice corner -> vertex index
  std::vector<GridVertex> grid;
  const int vCount = vx->voxelCount();
  for (int k = 0; k < vCount; k++) {
    CVX_Voxel* pV = vx->voxel(k);
    const int x = pV->indexX(), y = pV->indexY(), z = pV->indexZ();
    for (int i = 0; i < 6; i++) {  // each direction a face could be exposed in
      if (pV->adjacentVoxel((CVX_Voxel::linkDirection)i)) continue;
      for (int j = 0; j < 4; j++) {
        const int c = kFaceCorners[i][j];
        const int cx = x + ((c & 4) ? 1 : 0), cy = y + ((c & 2) ? 1 : 0), cz = z + ((c & 1) ? 1 : 0);
        auto it = vIndMap.find(grid_key(cx, cy, cz));
        int ind;
        if (it == vIndMap.end()) {
          ind = (int)grid.size();
          vIndMap.emplace(grid_key(cx, cy, cz), ind);
          grid.push_back({cx, cy, cz, ind});
          for (int m = 0; m < 3; m++) vertices.push_back(0);  // set by the first updateMesh
        } else {
          ind = it->second;
        }
        quads.push_back(ind);
      }
      quadVoxIndices.push_back(k);
    }
  }
  auto vertex_at = [&](int x, int y, int z) {
    auto it = vIndMap.find(grid_key(x, y, z));
    return it == vIndMap.end() ? -1 : it->second;
  };
  auto voxel_at = [&](int x, int y, int z) { return vx->voxel(x, y, z); };

  // vertex links and edges, visiting the vertices in lattice order (z, then y, then x)
  vertexLinks.assign(8 * grid.size(), -1);
  std::vector<GridVertex> order = grid;
  std::sort(order.begin(), order.end(), [](const GridVertex& a, const GridVertex& b) {
    if (a.z != b.z) return a.z < b.z;
    if (a.y != b.y) return a.y < b.y;
    return a.x < b.x;
  });
  for (const GridVertex& g : order) {
    const int x = g.x, y = g.y, z = g.z, thisInd = g.index;
    for (int i = 0; i < 8; i++) {  // the up to 8 voxels sharing this corner
      CVX_Voxel* pV = voxel_at(x - ((i & 4) ? 1 : 0), y - ((i & 2) ? 1 : 0), z - ((i & 1) ? 1 : 0));
      if (pV) vertexLinks[8 * thisInd + i] = pV->index();
    }
    for (int i = 0; i < 3; i++) {  // edges in +x, +y, +z where a voxel borders them
      const int isX = i == 0, isY = i == 1, isZ = i == 2;
      const int p2Ind = vertex_at(x + isX, y + isY, z + isZ);
      if (p2Ind == -1) continue;
      if (voxel_at(x, y, z) || voxel_at(x - isY, y - isX - isZ, z) || voxel_at(x - isY - isZ, y - isX - isZ, z - isX - isY) ||
          voxel_at(x - isZ, y, z - isX - isY)) {
        lines.push_back(thisInd);
        lines.push_back(p2Ind);
      }
    }
  }
  const int quadCount = (int)quads.size() / 4;
  quadColors.resize(quadCount * 3);
  quadNormals.resize(quadCount * 3);
  updateMesh();
}

void CVX_MeshRender::updateMesh(viewColoring colorScheme, CVoxelyze::stateInfoType stateType) {  // :141-218
  good = false;
  const int vCount = (int)vertices.size() / 3;
  if (vCount == 0) {
    good = true;
    return;
  }
  if (!vx->upload()) return;
  vxg_engine* eng = vx->impl()->eng;
  if (!uploaded) {
    if (vxg_mesh_topology(eng, vCount, vertexLinks.data(), (int)quads.size() / 4, quads.data())) return;
    uploaded = true;
  }
  if (vxg_mesh_update(eng, vertices.data(), quadNormals.empty() ? nullptr : quadNormals.data())) return;
  good = true;

  float minVal = 0, maxVal = 0;
  if (colorScheme == STATE_INFO) {
    maxVal = vx->stateInfo(stateType, CVoxelyze::MAX);
    minVal = vx->stateInfo(stateType, CVoxelyze::MIN);
    if (stateType == CVoxelyze::PRESSURE) {  // symmetric about zero
      maxVal = maxVal > -minVal ? maxVal : -minVal;
      minVal = -maxVal;
    }
  }
  const int qCount = (int)quads.size() / 4;
  for (int i = 0; i < qCount; i++) {
    CVX_Voxel* pV = vx->voxel(quadVoxIndices[i]);
    float r = 1.0f, g = 1.0f, b = 1.0f;
    float jetValue = -1.0f;
    switch (colorScheme) {
      case MATERIAL:
        r = ((float)pV->material()->red()) / 255.0f;
        g = ((float)pV->material()->green()) / 255.0f;
        b = ((float)pV->material()->blue()) / 255.0f;
        break;
      case FAILURE:
        if (pV->isFailed()) { g = 0.0f; b = 0.0f; }
        else if (pV->isYielded()) { b = 0.0f; }
        break;
      case STATE_INFO:
        switch (stateType) {
          case CVoxelyze::KINETIC_ENERGY: jetValue = pV->kineticEnergy() / maxVal; break;
          case CVoxelyze::STRAIN_ENERGY: case CVoxelyze::ENG_STRAIN: case CVoxelyze::ENG_STRESS:
            jetValue = linkMaxColorValue(pV, stateType) / maxVal;
            break;
          case CVoxelyze::DISPLACEMENT: jetValue = pV->displacementMagnitude() / maxVal; break;
          case CVoxelyze::PRESSURE: jetValue = 0.5 - pV->pressure() / (2 * maxVal); break;
          default: jetValue = 0;
        }
        break;
    }
    if (jetValue != -1.0f) {
      r = jetMapR(jetValue);
      g = jetMapG(jetValue);
      b = jetMapB(jetValue);
    }
    quadColors[i * 3] = r;
    quadColors[i * 3 + 1] = g;
    quadColors[i * 3 + 2] = b;
  }
}

float CVX_MeshRender::linkMaxColorValue(CVX_Voxel* pV, CVoxelyze::stateInfoType coloring) {  // :220-236
  float voxMax = -FLT_MAX;
  for (int i = 0; i < 6; i++) {
    float thisVal = -FLT_MAX;
    CVX_Link* pL = pV->link((CVX_Voxel::linkDirection)i);
    if (pL) {
      switch (coloring) {
        case CVoxelyze::STRAIN_ENERGY: thisVal = pL->strainEnergy(); break;
        case CVoxelyze::ENG_STRESS: thisVal = pL->axialStress(); break;
        case CVoxelyze::ENG_STRAIN: thisVal = pL->axialStrain(); break;
        default: thisVal = 0;
      }
    }
    if (thisVal > voxMax) voxMax = thisVal;
  }
  return voxMax;
}

void CVX_MeshRender::saveObj(const char* filePath) {  // :238-252
  std::ofstream ofile(filePath);
  ofile << "# OBJ file generated by Voxelyze\n";
  for (int i = 0; i < (int)(vertices.size() / 3); i++)
    ofile << "v " << vertices[3 * i] << " " << vertices[3 * i + 1] << " " << vertices[3 * i + 2] << "\n";
  for (int i = 0; i < (int)(quads.size() / 4); i++)
    ofile << "f " << quads[4 * i] + 1 << " " << quads[4 * i + 1] + 1 << " " << quads[4 * i + 2] + 1 << " "
          << quads[4 * i + 3] + 1 << "\n";
}

void CVX_MeshRender::glDraw() {}  // no OpenGL context in this library
