// dsc_noalloc.cu -- the tensor-core product on caller-owned device memory,
// with its scratch in a fixed static device array instead of cudaMalloc.
//
// Layout of the scratch (each part starts on a 256-byte boundary):
//   [0, 256)          error word of the tensor-core pipeline (int)
//   Bh, Bl            tf32 pair of B: Nc rows of round_up(Kd, 32) floats each
//   P                 S partial tiles of Nc x M floats (one per split of k)
// The error word must be zero when the GEMM kernel starts; every call
// clears it itself (cudaMemsetAsync on its stream) before its kernels run.
// Bh, Bl and P are written in full by each call before they are read, so
// nothing else needs a starting value.
#include <mutex>

#include "dsc_internal.h"
#include "dsc_tcgemm.h"
#include "depsolver_cuda.h"

namespace dsc {

constexpr size_t kScratchBytes = (size_t)DSC_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

// One copy per device, reserved when the module holding it is loaded on
// that device.
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// Address of g_scratch per device, looked up on the first call there.
static void *g_scratch_addr[kMaxDevices];
// Serialises calls: they share the one scratch of their device.
static std::mutex g_mu;

static size_t align256(size_t b) { return (b + 255) / 256 * 256; }

struct NoallocLayout {
    size_t ldbs, off_bh, off_bl, off_p, total;
};

static NoallocLayout layout_for(int M, int Nc, int Kd, int S)
{
    NoallocLayout L;
    L.ldbs = ((size_t)Kd + 31) / 32 * 32;
    const size_t bbytes = align256((size_t)Nc * L.ldbs * sizeof(float));
    L.off_bh = 256;
    L.off_bl = L.off_bh + bbytes;
    L.off_p = L.off_bl + bbytes;
    L.total = L.off_p + align256((size_t)S * Nc * (size_t)M * sizeof(float));
    return L;
}

static int check_device_ptr(const void *p, int dev, const char *name)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        set_error("dsc_tc_gemm_noalloc: %s is not a pointer CUDA knows", name);
        return kErrArg;
    }
    if (a.type == cudaMemoryTypeManaged) return kOk;
    if (a.type != cudaMemoryTypeDevice || a.device != dev) {
        set_error("dsc_tc_gemm_noalloc: %s must be device memory of the current device %d", name, dev);
        return kErrArg;
    }
    return kOk;
}

}  // namespace dsc

using namespace dsc;

// Y (M x Nc, row stride ldy, FP64) = A (M x Kd, FP32, row stride lda) *
// B^T (B: Nc x Kd, FP64, row stride ldb), all on the current device; the
// same 3xTF32 products, split of k and split order as dsc_tc_gemm.
extern "C" int dsc_tc_gemm_noalloc(int M, int Nc, int Kd, const float *A, size_t lda,
                                   const double *B, size_t ldb, double *Y, size_t ldy, int splits,
                                   void *stream)
{
    // shapes first: these checks touch no device
    if (M < 1 || Kd < 1 || Nc < 1 || Nc > 160) {
        set_error("dsc_tc_gemm_noalloc: unsupported shape M %d Nc %d Kd %d (M, Kd >= 1, 1 <= Nc <= 160)",
                  M, Nc, Kd);
        return kErrArg;
    }
    if (!A || !B || !Y || lda < (size_t)Kd || ldb < (size_t)Kd || ldy < (size_t)Nc) {
        set_error("dsc_tc_gemm_noalloc: null operand or row stride below the row length");
        return kErrArg;
    }
    if ((lda * sizeof(float)) % 16 || ((uintptr_t)A & 15)) {
        set_error("dsc_tc_gemm_noalloc: A needs a 16-byte aligned base and lda a multiple of 4");
        return kErrArg;
    }
    int S;
    if (splits > 0) {
        S = tc_gemm_splits_used(Kd, splits);
        if (layout_for(M, Nc, Kd, S).total > kScratchBytes) {
            set_error("dsc_tc_gemm_noalloc: M %d Nc %d Kd %d with %d splits needs %zu bytes of scratch; "
                      "the static scratch holds %zu",
                      M, Nc, Kd, S, layout_for(M, Nc, Kd, S).total, kScratchBytes);
            return kErrArg;
        }
    } else {
        // the split count dsc_tc_gemm would pick, lowered until it fits
        S = tc_gemm_splits_for(M, Kd);
        while (S > 1 && layout_for(M, Nc, Kd, S).total > kScratchBytes)
            S = tc_gemm_splits_used(Kd, S - 1);
        if (layout_for(M, Nc, Kd, S).total > kScratchBytes) {
            set_error("dsc_tc_gemm_noalloc: M %d Nc %d Kd %d needs %zu bytes of scratch even unsplit; "
                      "the static scratch holds %zu",
                      M, Nc, Kd, layout_for(M, Nc, Kd, 1).total, kScratchBytes);
            return kErrArg;
        }
    }
    const NoallocLayout L = layout_for(M, Nc, Kd, S);

    std::lock_guard<std::mutex> lk(g_mu);
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        set_error("no CUDA device available");
        return kErrCuda;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("dsc_tc_gemm_noalloc: device %d above the supported %d", dev, kMaxDevices);
        return kErrArg;
    }
    DSC_TRY(check_device_ptr(A, dev, "A"));
    DSC_TRY(check_device_ptr(B, dev, "B"));
    DSC_TRY(check_device_ptr(Y, dev, "Y"));
    if (!g_scratch_addr[dev]) DSC_CUDA(cudaGetSymbolAddress(&g_scratch_addr[dev], g_scratch));
    unsigned char *base = (unsigned char *)g_scratch_addr[dev];
    int *err = (int *)base;
    float *Bh = (float *)(base + L.off_bh);
    float *Bl = (float *)(base + L.off_bl);
    float *P = (float *)(base + L.off_p);

    cudaStream_t st = (cudaStream_t)stream;
    DSC_CUDA(cudaMemsetAsync(err, 0, sizeof(int), st));
    DSC_TRY(split_rows(B, ldb, Nc, Kd, Bh, Bl, L.ldbs, st));
    DSC_TRY(tc_gemm_3xtf32(A, nullptr, lda, Bh, Bl, L.ldbs, M, Nc, Kd, P, (size_t)M, S, err, st));
    DSC_TRY(sum_splits(P, S, (size_t)M * Nc, (size_t)M, M, Nc, Y, ldy, st));
    int herr = 0;
    DSC_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, st));
    DSC_CUDA(cudaStreamSynchronize(st));
    if (herr) {
        set_error("tensor-core GEMM: a pipeline wait gave up (code %d)", herr);
        return kErrCuda;
    }
    return kOk;
}
