// 2D row passes (float, radix 8) with plain twiddles: the momentum form's variants.
#define QSG_PLAIN_UNIT 1
#include "qsg_row_f32b.cu"
