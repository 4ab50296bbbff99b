// The reference's scene-file calls compiled against this repository's headers: saveJSON, the
// CVoxelyze(const char*) constructor and loadJSON (include/Voxelyze.h:70-78 of the reference).
// Host-only: no time step runs.  Prints what the Python test checks.
#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>

#include "Voxelyze.h"

static std::string slurp(const char* p) {
  std::ifstream f(p);
  std::stringstream s;
  s << f.rdbuf();
  return s.str();
}

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  CVoxelyze Vx(0.005);
  CVX_Material* pMaterial = Vx.addMaterial(1000000, 1000);
  pMaterial->setPoissonsRatio(0.3f);
  Vx.setVoxel(pMaterial, 0, 0, 0)->external()->setFixedAll();
  Vx.setVoxel(pMaterial, 1, 0, 0);
  Vx.setVoxel(pMaterial, 2, 0, 0)->external()->setForce(0, 0, -1);
  if (!Vx.saveJSON(argv[1])) return 3;
  CVoxelyze Vx2(argv[1]);  // the JSON constructor
  if (!Vx2.saveJSON(argv[2])) return 4;
  CVoxelyze Vx3;
  bool loaded = Vx3.loadJSON(argv[2]);
  std::printf("voxels %d links %d materials %d nu %.7g loaded %d same %d\n", Vx2.voxelCount(), Vx2.linkCount(),
              Vx2.materialCount(), Vx3.material(0)->poissonsRatio(), loaded ? 1 : 0,
              slurp(argv[1]) == slurp(argv[2]) ? 1 : 0);
  return 0;
}
