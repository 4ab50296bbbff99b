// The reference README's usage example (README.md:21-44) and the query calls its tests use,
// compiled unchanged against this repository's headers.  Prints the final state so the Python
// test can compare it with the oracle.
#include <cstdio>

#include "Voxelyze.h"

int main() {
  CVoxelyze Vx(0.005);                                      // 5mm voxels
  CVX_Material* pMaterial = Vx.addMaterial(1000000, 1000);  // E = 1 MPa, rho = 1000 kg/m^3
  CVX_Voxel* Voxel1 = Vx.setVoxel(pMaterial, 0, 0, 0);
  CVX_Voxel* Voxel2 = Vx.setVoxel(pMaterial, 1, 0, 0);
  CVX_Voxel* Voxel3 = Vx.setVoxel(pMaterial, 2, 0, 0);
  (void)Voxel2;
  Voxel1->external()->setFixedAll();
  Voxel3->external()->setForce(0, 0, -1);
  for (int i = 0; i < 100; i++) Vx.doTimeStep();
  for (int i = 0; i < Vx.voxelCount(); i++) {
    Vec3D<> p = Vx.voxel(i)->position();
    Quat3D<> q = Vx.voxel(i)->orientation();
    std::printf("%d %.17g %.17g %.17g %.17g %.17g %.17g %.17g\n", i, p.x, p.y, p.z, q.w, q.x, q.y, q.z);
  }
  std::printf("links %d small %d strain %.9g\n", Vx.linkCount(), Vx.link(0)->isSmallAngle() ? 1 : 0,
              Vx.link(0)->axialStrain());
  std::printf("ke %.9g disp %.9g\n", Vx.stateInfo(CVoxelyze::KINETIC_ENERGY, CVoxelyze::TOTAL),
              Vx.stateInfo(CVoxelyze::DISPLACEMENT, CVoxelyze::MAX));
  return 0;
}
