// Specialised cascade variants: 256x256 inputs at J=4 (padded 288).
#include "ct_cascade.cuh"
#include "bwd.cuh"
KYM_CT_VARIANT(288, 288, 18, 18, 4, false, 512)
KYM_CT_FOLD(288, 288, 18, 18, 4, false, 512, 0)
KYM_CT_FOLD(288, 288, 18, 18, 4, false, 512, 1)
KYM_CT_VARIANT(144, 144, 18, 18, 1, false, 512)
KYM_CT_FOLD(144, 144, 18, 18, 1, false, 512, 2)
KYM_CT_VARIANT(72, 72, 18, 18, 1, false, 512)
KYM_CT_FOLD(72, 72, 18, 18, 1, false, 512, 2)
KYM_CT_FOLD(72, 72, 18, 18, 1, false, 512, 4)
KYM_CT_VARIANT(36, 36, 18, 18, 1, false, 512)
KYM_CT_FOLD(36, 36, 18, 18, 1, false, 512, 2)
KYM_CT_FOLD(36, 36, 18, 18, 1, false, 512, 4)
KYM_CT_FOLD(36, 36, 18, 18, 1, false, 512, 8)
KYM_BWD_VARIANT(288, 288, 18, 18, 4, false, 512)
KYM_BWD_VARIANT(144, 144, 18, 18, 1, false, 512)
KYM_BWD_VARIANT(72, 72, 18, 18, 1, false, 512)
KYM_BWD_VARIANT(36, 36, 18, 18, 1, false, 512)
