// batched_study.cu -- instantiations of the batched step kernel (batched_kernel.cuh) for
// the precision study: reference arithmetic with compensated (Kahan) float32
// accumulation, with plain float32 atomics, and the float64 build.  Compiled without
// multiply-add contraction and with IEEE division and square root, as batched_ref.cu.
#include "batched_kernel.cuh"

namespace ffsrl {

using namespace bk;

kern_f pick_ref_study(int accumulation, int block, int mode) {
    if (accumulation == FFSRL_ACC_KAHAN) {
#define PK(B, M) if (block == B && mode == M) return k_batched<AccKahan, B, M, false, 0, true>;
        PK(256, 0) PK(512, 0) PK(1024, 0) PK(256, 1) PK(512, 1) PK(256, 2)
#undef PK
    }
    if (accumulation == FFSRL_ACC_ATOMIC) {
#define PK(B, M) if (block == B && mode == M) return k_batched<AccAtomic, B, M, false, 0, true>;
        PK(256, 0) PK(512, 0) PK(1024, 0) PK(256, 1) PK(512, 1) PK(256, 2)
#undef PK
    }
    return nullptr;
}

kern_d pick_ref_f64(int block, int mode) {
    if (block == 256 && mode == 0) return k_batched<AccF64, 256, 0, false, 0, true>;
    if (block == 256 && mode == 2) return k_batched<AccF64, 256, 2, false, 0, true>;
    return nullptr;
}

}  // namespace ffsrl
