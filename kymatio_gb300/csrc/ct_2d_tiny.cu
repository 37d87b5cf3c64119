// Specialised cascade variants: padded sizes 40 and 20 with a 10x10 low-pass.
#include "ct_cascade.cuh"
#include "bwd.cuh"
KYM_CT_VARIANT(40, 40, 10, 10, 1, false, 512)
KYM_CT_FOLD(40, 40, 10, 10, 1, false, 512, 0)
KYM_CT_FOLD(40, 40, 10, 10, 1, false, 512, 1)
KYM_CT_FOLD(40, 40, 10, 10, 1, false, 512, 2)
KYM_CT_FOLD(40, 40, 10, 10, 1, false, 512, 4)
KYM_CT_VARIANT(20, 20, 10, 10, 1, false, 512)
KYM_CT_FOLD(20, 20, 10, 10, 1, false, 512, 2)
KYM_CT_FOLD(20, 20, 10, 10, 1, false, 512, 4)
KYM_CT_FOLD(20, 20, 10, 10, 1, false, 512, 8)
KYM_BWD_VARIANT(40, 40, 10, 10, 1, false, 512)
KYM_BWD_VARIANT(20, 20, 10, 10, 1, false, 512)
