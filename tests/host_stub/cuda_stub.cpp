// Test infrastructure only: a host-memory stand-in for the parts of the CUDA
// runtime that the transfer plan's host code calls, so that the CPU tests can
// build csrc/transfer.cpp into a library of its own and check its host logic
// (the classification, the nested rule's lines and points, the pairing's
// support elements, the refusals) against the oracle without a GPU. "Device"
// buffers are host allocations; every host-to-device copy is logged with a
// copy of its bytes; kernel launches do nothing. The product never links it.
#include <cuda_runtime_api.h>

#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/twoldg.h"
#include "../../treewaveoldg.jl_gb300/csrc/transfer.h"

namespace {
int g_shape[5] = {3, 3, 2, 0, 1};   // D, P, E, prec, nblocks
std::string g_error;
std::vector<std::vector<unsigned char>> g_uploads;
}  // namespace

extern "C" {

cudaError_t cudaMalloc(void** p, size_t n) {
    *p = std::calloc(1, n ? n : 1);
    return *p ? cudaSuccess : cudaErrorMemoryAllocation;
}
cudaError_t cudaFree(void* p) {
    std::free(p);
    return cudaSuccess;
}
cudaError_t cudaHostAlloc(void** p, size_t n, unsigned int) { return cudaMalloc(p, n); }
cudaError_t cudaFreeHost(void* p) { return cudaFree(p); }
cudaError_t cudaMemcpy(void* d, const void* s, size_t n, cudaMemcpyKind kind) {
    std::memcpy(d, s, n);
    if (kind == cudaMemcpyHostToDevice) {
        const unsigned char* b = static_cast<const unsigned char*>(s);
        g_uploads.emplace_back(b, b + n);
    }
    return cudaSuccess;
}
cudaError_t cudaMemcpyAsync(void* d, const void* s, size_t n, cudaMemcpyKind kind, cudaStream_t) {
    return cudaMemcpy(d, s, n, kind);
}
cudaError_t cudaStreamSynchronize(cudaStream_t) { return cudaSuccess; }
cudaError_t cudaDeviceSynchronize(void) { return cudaSuccess; }
cudaError_t cudaEventSynchronize(cudaEvent_t) { return cudaSuccess; }
const char* cudaGetErrorString(cudaError_t) { return "host stand-in"; }
cudaError_t cudaDeviceGetStreamPriorityRange(int* least, int* greatest) {
    *least = 0;
    *greatest = -1;
    return cudaSuccess;
}
cudaError_t cudaStreamCreateWithPriority(cudaStream_t* s, unsigned int, int) {
    *s = reinterpret_cast<cudaStream_t>(std::malloc(1));
    return cudaSuccess;
}
cudaError_t cudaStreamDestroy(cudaStream_t s) {
    std::free(s);
    return cudaSuccess;
}
cudaError_t cudaEventCreateWithFlags(cudaEvent_t* e, unsigned int) {
    *e = reinterpret_cast<cudaEvent_t>(std::malloc(1));
    return cudaSuccess;
}
cudaError_t cudaEventDestroy(cudaEvent_t e) {
    std::free(e);
    return cudaSuccess;
}
cudaError_t cudaEventRecord(cudaEvent_t, cudaStream_t) { return cudaSuccess; }
cudaError_t cudaStreamWaitEvent(cudaStream_t, cudaEvent_t, unsigned int) { return cudaSuccess; }

// the stand-in's own controls
void stub_set_shape(int D, int P, int E, int prec, int nblocks) {
    const int v[5] = {D, P, E, prec, nblocks};
    std::memcpy(g_shape, v, sizeof v);
}
const char* stub_last_error() { return g_error.c_str(); }
void stub_reset_uploads() { g_uploads.clear(); }
int64_t stub_nuploads() { return (int64_t)g_uploads.size(); }
int64_t stub_upload_size(int64_t i) { return (int64_t)g_uploads[i].size(); }
const void* stub_upload_data(int64_t i) { return g_uploads[i].data(); }

}  // extern "C"

namespace twoldg {
int static_rhs_fail(int code, const std::string& msg) {
    g_error = msg;
    return code;
}
bool problem_shape(twoldg_problem*, int* D, int* P, int* E, int* prec, int64_t* nblocks, cudaStream_t* stream) {
    *D = g_shape[0];
    *P = g_shape[1];
    *E = g_shape[2];
    *prec = g_shape[3];
    *nblocks = g_shape[4];
    *stream = nullptr;
    return true;
}
cudaError_t launch_projection(const TransferLaunch&, cudaStream_t, cudaStream_t, cudaStream_t) { return cudaSuccess; }
cudaError_t launch_points(const TransferLaunch&, void*, int64_t, cudaStream_t) { return cudaSuccess; }
cudaError_t launch_average(const AverageLaunch&, cudaStream_t) { return cudaSuccess; }
cudaError_t launch_pairing_moments(const PairingLaunch&, cudaStream_t) { return cudaSuccess; }
cudaError_t launch_pairing_dot(const PairingLaunch&, cudaStream_t) { return cudaSuccess; }
}  // namespace twoldg
