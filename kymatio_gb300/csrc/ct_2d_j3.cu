// Specialised cascade variants: 256x256 inputs at J=3 (padded 272).
#include "ct_cascade.cuh"
#include "bwd.cuh"
KYM_CT_VARIANT(272, 272, 34, 34, 4, false, 512)
KYM_CT_FOLD(272, 272, 34, 34, 4, false, 512, 0)
KYM_CT_FOLD(272, 272, 34, 34, 4, false, 512, 1)
KYM_CT_VARIANT(136, 136, 34, 34, 1, false, 640)
KYM_CT_FOLD(136, 136, 34, 34, 1, false, 640, 2)
KYM_CT_VARIANT(68, 68, 34, 34, 1, false, 512)
KYM_CT_FOLD(68, 68, 34, 34, 1, false, 512, 2)
KYM_CT_FOLD(68, 68, 34, 34, 1, false, 512, 4)
KYM_BWD_VARIANT(272, 272, 34, 34, 4, false, 512)
KYM_BWD_VARIANT(136, 136, 34, 34, 1, false, 512)
KYM_BWD_VARIANT(68, 68, 34, 34, 1, false, 512)
