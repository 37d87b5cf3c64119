// Specialised 1-D cascade variants: padded length 16384 down to 256 with a
// 256-sample low-pass (8192-sample signals, T=64).
#include "ct_cascade.cuh"
#include "bwd.cuh"
KYM_CT_VARIANT(1, 16384, 1, 256, 1, true, 512)
KYM_CT_VARIANT(1, 8192, 1, 256, 1, true, 512)
KYM_CT_VARIANT(1, 4096, 1, 256, 1, true, 512)
KYM_CT_VARIANT(1, 2048, 1, 256, 1, true, 512)
KYM_CT_VARIANT(1, 1024, 1, 256, 1, true, 512)
KYM_CT_VARIANT(1, 512, 1, 256, 1, true, 512)
KYM_CT_VARIANT(1, 256, 1, 256, 1, true, 512)
KYM_BWD_VARIANT(1, 16384, 1, 256, 1, true, 512)
KYM_BWD_VARIANT(1, 8192, 1, 256, 1, true, 512)
KYM_BWD_VARIANT(1, 4096, 1, 256, 1, true, 512)
KYM_BWD_VARIANT(1, 2048, 1, 256, 1, true, 512)
KYM_BWD_VARIANT(1, 1024, 1, 256, 1, true, 512)
KYM_BWD_VARIANT(1, 512, 1, 256, 1, true, 512)
KYM_BWD_VARIANT(1, 256, 1, 256, 1, true, 512)
