// Direct access to the engine's predicates, for callers that want the exact
// orientation / in-circle signs of their own points, and for testing the
// predicates in isolation: the host versions (the same source as the device
// versions, compiled for the CPU) and a batched device evaluation.
#include <cuda_runtime.h>

#include "predicates.cuh"
#include "qdt_gpu.h"

namespace qdtg {

// kind 0: orient2d on 6 doubles per item; kind 1: in-circle on 8 doubles.
// mode 0: full predicate; 1: float pre-filter only (0 = undecided);
// 2: exact evaluation only.
QDT_HD inline int eval_one(int kind, int mode, const double* v, size_t i)
{
    int s;
    if (kind == 0)
    {
        const double* q = v + 6 * i;
        if (mode == 1)
            s = orient2d_f32(sub_rn(q[0], q[4]), sub_rn(q[1], q[5]), sub_rn(q[2], q[4]), sub_rn(q[3], q[5]));
        else if (mode == 2)
            s = orient2d_exact(q);
        else
            s = orient2d_sign(q[0], q[1], q[2], q[3], q[4], q[5]);
    }
    else
    {
        const double* q = v + 8 * i;
        if (mode == 1)
            s = incircle_f32(sub_rn(q[0], q[6]), sub_rn(q[1], q[7]), sub_rn(q[2], q[6]), sub_rn(q[3], q[7]),
                sub_rn(q[4], q[6]), sub_rn(q[5], q[7]));
        else if (mode == 2)
            s = incircle_exact(q);
        else
            s = incircle_sign(q[0], q[1], q[2], q[3], q[4], q[5], q[6], q[7]);
    }
    return s;
}

__global__ void k_eval_pred(int kind, int mode, const double* __restrict__ v, size_t count, int8_t* __restrict__ out)
{
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) out[i] = (int8_t)eval_one(kind, mode, v, i);
}

}  // namespace qdtg

extern "C" {

QDT_API int qdtg_orient2d(const double* a, const double* b, const double* c)
{
    return qdtg::orient2d_sign(a[0], a[1], b[0], b[1], c[0], c[1]);
}

QDT_API int qdtg_incircle(const double* a, const double* b, const double* c, const double* d)
{
    return qdtg::incircle_sign(a[0], a[1], b[0], b[1], c[0], c[1], d[0], d[1]);
}

QDT_API int qdtg_eval_predicates(int kind, int mode, int on_device, const double* coords, size_t count, int8_t* out)
{
    if (count == 0) return 0;
    if (!coords || !out || kind < 0 || kind > 1 || mode < 0 || mode > 2) return -2;
    if (!on_device)
    {
        for (size_t i = 0; i < count; ++i) out[i] = (int8_t)qdtg::eval_one(kind, mode, coords, i);
        return 0;
    }
    const size_t per = kind == 0 ? 6 : 8;
    double*      dv = nullptr;
    int8_t*      dout = nullptr;
    int          rc = 0;
    if (cudaMalloc(&dv, per * count * sizeof(double)) != cudaSuccess ||
        cudaMalloc(&dout, count) != cudaSuccess)
        rc = -10;
    if (!rc && cudaMemcpy(dv, coords, per * count * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) rc = -11;
    if (!rc)
    {
        qdtg::k_eval_pred<<<(unsigned)((count + 255) / 256), 256>>>(kind, mode, dv, count, dout);
        if (cudaMemcpy(out, dout, count, cudaMemcpyDeviceToHost) != cudaSuccess) rc = -11;
    }
    cudaGetLastError();
    if (dv) cudaFree(dv);
    if (dout) cudaFree(dout);
    return rc;
}

}  // extern "C"
