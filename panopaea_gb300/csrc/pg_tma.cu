// pg_tma.cu -- host side of pg_tma.cuh: tensor-map encoding through the
// driver entry point (no link-time dependency on libcuda).
#include <mutex>

#include "pg_tma.cuh"

namespace pg {

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
        else
            cudaGetLastError();
    });
    return fn;
}

bool encode_map_3d(CUtensorMap* map, const void* base, int elem, i64 w, i64 h, i64 d, int bx, int by) {
    auto fn = encode_fn();
    if (!fn || !base) return false;
    if (((uintptr_t)base & 15) || ((w * elem) & 15) || ((bx * elem) & 15)) return false;
    if (w > 0x7fffffff || h > 0x7fffffff || d > 0x7fffffff || bx > 256 || by > 256) return false;
    CUtensorMapDataType dt;
    if (elem == 4) dt = CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    else if (elem == 1) dt = CU_TENSOR_MAP_DATA_TYPE_UINT8;
    else return false;
    const cuuint64_t dims[3] = {(cuuint64_t)w, (cuuint64_t)h, (cuuint64_t)d};
    const cuuint64_t strides[2] = {(cuuint64_t)(w * elem), (cuuint64_t)(w * h * elem)};
    const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    const CUresult r = fn(map, dt, 3, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

}  // namespace pg

extern "C" int pg_debug_set_stage_wait_polls(uint32_t polls) {
    int rc = pg::set_stage_wait_polls_spmv(polls);
    if (rc == PG_OK) rc = pg::set_stage_wait_polls_mg(polls);
    return rc;
}

extern "C" uint32_t pg_debug_stage_wait_polls_default(void) { return pg::kMbarSpinLimit; }
