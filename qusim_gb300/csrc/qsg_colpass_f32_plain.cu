// 2D column passes (float) with plain twiddles: the momentum form's variants.
#define QSG_PLAIN_UNIT 1
#include "qsg_colpass_f32.cu"
