// batched_ref.cu -- the reference-arithmetic instantiations of the batched step kernel
// (batched_kernel.cuh, EX = true) with fixed-point accumulation.  This unit is compiled
// without multiply-add contraction and with IEEE division and square root, so every
// constraint's corrections are the ones the reference kernel's expressions give.
#include "batched_kernel.cuh"

namespace ffsrl {

using namespace bk;

kern_f pick_ref_fixed(int block, int mode, int prefetch, unsigned flags) {
    if (flags == kLiverFlags && mode == 0 && prefetch != 2) {
        if (block == 256) return k_batched<AccFixed, 256, 0, false, kLiverFlags, true>;
        if (block == 512) return k_batched<AccFixed, 512, 0, false, kLiverFlags, true>;
        if (block == 640) return k_batched<AccFixed, 640, 0, false, kLiverFlags, true>;
        if (block == 768) return k_batched<AccFixed, 768, 0, false, kLiverFlags, true>;
        if (block == 1024) return k_batched<AccFixed, 1024, 0, false, kLiverFlags, true>;
    }
    if (flags == kLiverFlags && mode == 0 && prefetch == 2) {
        if (block == 512) return k_batched<AccFixed, 512, 0, true, kLiverFlags, true>;
        if (block == 640) return k_batched<AccFixed, 640, 0, true, kLiverFlags, true>;
        return nullptr;
    }
    if (prefetch == 2) {
        if (mode == 0 && block == 512) return k_batched<AccFixed, 512, 0, true, 0, true>;
        if (mode == 0 && block == 640) return k_batched<AccFixed, 640, 0, true, 0, true>;
        return nullptr;
    }
#define PK(B, M) if (block == B && mode == M) return k_batched<AccFixed, B, M, false, 0, true>;
    PK(128, 0) PK(256, 0) PK(512, 0) PK(640, 0) PK(768, 0) PK(1024, 0)
    PK(256, 1) PK(512, 1) PK(1024, 1)
    PK(256, 2) PK(512, 2)
#undef PK
    return nullptr;
}

}  // namespace ffsrl
