// Born-series kernels, complex128 instantiations.
#include "qsg_born_inst.cuh"

namespace qsg {

QSG_BORN_INSTANTIATE(double)

}  // namespace qsg
