// twoldg_rhs_static: the right-hand side with no device allocation.
//
// Some callers cannot call cudaMalloc: a host that hands the GPU to the
// library only through buffers it manages itself (a fixed arena, a memory
// pool that forbids growth, or an embedding runtime whose allocator the
// library must not bypass). For them this entry point evaluates
// du = (v, sum_d D_d D_d u) for a forest given by its descriptor, like
// twoldg_rhs, but keeps its scratch -- the work-item table, the per-face
// exports of u and the coarse-fine ghost planes -- in one file-scope
// __device__ array of kScratchBytes, which every GPU that loads the library
// holds until the process exits. The caller still passes u and du.
//
// Set-up: the first call on a device (with that device current) looks up
// the array's device address with cudaGetSymbolAddress and caches it per
// device, so that first call should come before any stream capture. The
// cached address belongs to the device's primary context: after a
// cudaDeviceReset the array moves and the cache is stale, so a process that
// resets a device must not call this entry point on it again. Every
// call shares the one array per device and overwrites it; nothing in it has
// to start at zero (each call writes every word it later reads), but calls
// whose work overlaps on the GPU race on it, so a caller serialises them.
#include <cuda_runtime.h>

#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/twoldg.h"
#include "mesh.h"
#include "ops.h"
#include "tables.h"

namespace {

constexpr size_t kScratchBytes = size_t(16) << 20;  // 16 MiB per device
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_static_scratch[kScratchBytes];

std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {};

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

}  // namespace

namespace twoldg {
int static_rhs_fail(int code, const std::string& msg);
bool static_rhs_tables(int P, const ElementTables<double>** t64, const ElementTables<float>** t32);
}  // namespace twoldg

extern "C" int twoldg_rhs_static(const twoldg_desc* desc, void* du, const void* u, double t, void* stream) {
    using namespace twoldg;
    (void)t;
    if (!desc || !du || !u) return static_rhs_fail(TWOLDG_EINVAL, "desc, du and u must not be NULL");
    if (du == u) return static_rhs_fail(TWOLDG_EINVAL, "du and u must not alias: the right-hand side never writes u");
    // Only the flat brick: the flat kernels read a neighbour's face plane as it
    // lies, so a metric or an explicit face table (oriented glues, boundary
    // faces) would be read wrongly. Checked before any CUDA call.
    if (desc->coef || desc->metric != 0)
        return static_rhs_fail(TWOLDG_EUNSUP, "twoldg_rhs_static serves flat problems (coef = NULL, metric = 0)");
    if (desc->face_nb || desc->face_code)
        return static_rhs_fail(TWOLDG_EUNSUP, "twoldg_rhs_static serves a brick of roots, not an explicit face "
                                              "table (face_nb = NULL)");
    Mesh m;
    std::string err;
    if (!build_mesh(*desc, m, err)) return static_rhs_fail(TWOLDG_EINVAL, err);
    const int prec = desc->precision;
    if (prec != TWOLDG_F64 && prec != TWOLDG_F32 && prec != TWOLDG_F32C)
        return static_rhs_fail(TWOLDG_EINVAL, "precision must be TWOLDG_F64, TWOLDG_F32 or TWOLDG_F32C");
    const size_t w = prec == TWOLDG_F64 ? 8 : 4;
    size_t F = 1;
    for (int k = 0; k < m.D - 1; ++k) F *= m.N;
    const size_t nslots = (size_t)m.nblocks * 2 * m.D;
    const size_t face_bytes = align256(nslots * F * w);
    const size_t items_bytes = align256(m.items.size() * sizeof(BlockItem));
    const size_t cf_bytes = align256(m.cf.size() * sizeof(CfFace));
    const size_t ndense = m.cf.empty() ? 0 : 3;
    const size_t need = items_bytes + cf_bytes + 2 * face_bytes + ndense * face_bytes;
    if (need > kScratchBytes)
        return static_rhs_fail(TWOLDG_EINVAL, "the forest needs " + std::to_string(need) +
                                                  " bytes of scratch and twoldg_rhs_static holds at most " +
                                                  std::to_string(kScratchBytes) +
                                                  " (16 MiB): use twoldg_rhs, whose problem allocates its own");
    const ElementTables<double>* t64;
    const ElementTables<float>* t32;
    if (!static_rhs_tables(m.P, &t64, &t32))
        return static_rhs_fail(TWOLDG_EUNSUP, "element order P = " + std::to_string(m.P) + " is not built (1..8)");
    Ops* ops = nullptr;
    if (m.D == 1) ops = make_ops_d1(prec, m.P, *t64, *t32);
    if (m.D == 2) ops = make_ops_d2(prec, m.P, *t64, *t32);
    if (m.D == 3) ops = make_ops_d3(prec, m.P, *t64, *t32);
    if (!ops) return static_rhs_fail(TWOLDG_EUNSUP, "no kernels for this order");
    if (ops->stage_smem(m.E) > 227 * 1024) {
        delete ops;
        return static_rhs_fail(TWOLDG_EUNSUP, "block too large for one CTA's shared memory");
    }
    std::unique_ptr<Ops> own(ops);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return static_rhs_fail(TWOLDG_ECUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return static_rhs_fail(TWOLDG_EUNSUP, "device ordinal beyond 64");
    void* base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        if (!g_scratch_ptr[dev]) {
            void* p = nullptr;
            e = cudaGetSymbolAddress(&p, g_static_scratch);
            if (e != cudaSuccess)
                return static_rhs_fail(TWOLDG_ECUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
            g_scratch_ptr[dev] = p;
        }
        base = g_scratch_ptr[dev];
    }
    cudaStream_t s = (cudaStream_t)stream;
    unsigned char* p = (unsigned char*)base;
    BlockItem* d_items = (BlockItem*)p;
    p += items_bytes;
    CfFace* d_cf = (CfFace*)p;
    p += cf_bytes;
    void* fu = p;
    p += face_bytes;
    void* fog = p;
    p += face_bytes;
    void* ugd = ndense ? (void*)p : nullptr;
    void* gfd = ndense ? (void*)(p + face_bytes) : nullptr;
    void* ggd = ndense ? (void*)(p + 2 * face_bytes) : nullptr;
    int rc = TWOLDG_OK;
    auto ck = [&](cudaError_t ce, const char* what) {
        if (ce != cudaSuccess && rc == TWOLDG_OK)
            rc = static_rhs_fail(TWOLDG_ECUDA, std::string(what) + ": " + cudaGetErrorString(ce));
        return ce == cudaSuccess;
    };
    if (ck(cudaMemcpyAsync(d_items, m.items.data(), m.items.size() * sizeof(BlockItem), cudaMemcpyHostToDevice, s),
           "cudaMemcpyAsync(items)") &&
        (m.cf.empty() || ck(cudaMemcpyAsync(d_cf, m.cf.data(), m.cf.size() * sizeof(CfFace),
                                            cudaMemcpyHostToDevice, s), "cudaMemcpyAsync(cf)")) &&
        ck(ops->export_faces(d_items, m.nblocks, m.E, u, fu, fog, s), "export_faces") &&
        ck(ops->cf_ghosts(d_cf, (int)m.cf.size(), m.E, fu, fog, ugd, gfd, ggd, s), "cf_ghosts")) {
        StagePtrs sp{};
        sp.u = const_cast<void*>(u);
        sp.du = du;
        sp.fu_in = fu;
        sp.fog_in = fog;
        sp.ugd = ugd;
        sp.ggd = ggd;
        ck(ops->stage(d_items, m.nblocks, m.E, 0, 0, sp, 0, s), "stage");
    }
    // The host tables the copies read are staged before cudaMemcpyAsync returns
    // (pageable source), and the kernels took their tables by value, so both
    // may go now (with `own`); the work itself stays queued on `stream`.
    return rc;
}
