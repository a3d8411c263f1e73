// 3D passes, complex128 instantiations.
#include "qsg_evolve3d_inst.cuh"

namespace qsg {

QSG_3D_INSTANTIATE(double)

}  // namespace qsg
