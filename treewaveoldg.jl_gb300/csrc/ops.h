// Host-side interface to the templated kernels: one Ops object per
// (precision, dimension, order), created at problem set-up. Pointers are
// device pointers of the problem's precision; sizes are in words.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "kernels_types.h"
#include "tables.h"

namespace twoldg {

enum Precision : int { PREC_F64 = 0, PREC_F32 = 1, PREC_F32C = 2 };

struct StagePtrs {
    void* u;
    void* y;
    void* acc;
    void* comp;
    void* du;
    const void* fu_in;
    const void* fog_in;
    void* fu_out;
    void* fog_out;
    const void* ugd;
    const void* ggd;
    const void* rk;    // per problem 4 RK coefficients in the field type
    double* partial;
    const void* coef;  // diagonal metric node values (NULL: flat)
    const void* trm;   // per-line truncation pairs (NULL: the element's)
    const void* trd;
    // coarse-fine faces (NULL: none, or their ghost planes ugd and ggd are
    // filled by the caller); cfidx gives per face slot the face's index in cf
    // (-1: none). The 3D register-line kernel reads ugd, ggd and its own part
    // gsd as the previous stage's epilogues wrote them and writes the next
    // stage's into the *_out planes; the other kernels have ugd and ggd
    // filled by a launch of their own before the stage kernel.
    const CfFace* cf;
    const int* cfidx;
    int ncf;
    const void* gsd;
    void* ugd_out;
    void* ggd_out;
    void* gsd_out;
    // the register-line stage kernels as programmatic dependent launches
    // (each may become resident while the kernel before it finishes)
    int pdl;
};

// Buffers and data of the full-metric passes (fullmetric.cuh).
struct FmPtrs {
    void* u;
    void* y;
    void* acc;
    void* comp;
    void* du;
    const void* fu_in;
    void* fu_out;
    void* V;
    void* fv;
    const void* coef;
    const void* M;      // sqrt(g) g^de per node, 6 per node (00, 11, 22, 01, 02, 12)
    const void* rk;
    const double* tinfo;
    const double* bnd_x;
    double wave_k[3];
    double wave_phi;
    const int* eslot;
    const void* ew;
    const void* echol;
    double* partial;
    int boundary;       // 0 Dirichlet plane wave, 1 radiative, 2 the caller's Dirichlet values
    double kappa;
    double inv_r;
    const int* fslot;   // factored truncation (fullmetric.cuh)
    const int* fradial;
    const void* frm;
    const void* frd;
    const int* faslot;
    const void* faw;
    const void* fachol;
    const int* bidx;    // boundary kind 2: per face slot its boundary face index (-1 inside)
    const BoundaryTable* btab;
    const void* ugd;    // coarse-fine faces (a refined brick patch): u's ghosts per slot (N^2)
    const void* vgd;    // and V's, (3, N^2) per slot
    int pdl;            // the register-line passes as programmatic dependent launches
};

// A launch layout of the stage kernel. kernel: 0 the shape's default, 1 the
// register-line 3D kernel, 2 the fixed-shape kernel, 3 the run-time-shape
// kernel; threads: threads per CTA of kernel 3 (0: by block size); waves: 0
// one CTA per block, k > 0 at most k times the CTAs the device holds at once,
// each CTA looping over blocks (so that its prefetch of the next block pays).
struct Launch {
    int kernel;
    int threads;
    int waves;
};

class Ops {
public:
    virtual ~Ops() {}
    // bytes of dynamic shared memory the stage kernel needs for E elements per dim
    virtual size_t stage_smem(int E) const = 0;
    // the stage kernel's launch layout (the autotuner sets it, before a graph is captured)
    virtual void set_launch(const Launch& l, int E, bool flat) = 0;
    virtual Launch launch() const = 0;
    // the layouts worth timing for blocks of E elements per dimension; flat:
    // no metric coefficients. Returns how many were written (at most max).
    virtual int launch_candidates(int E, bool flat, Launch* out, int max) const = 0;
    virtual cudaError_t export_faces(const BlockItem* items, int nitems, int E, const void* u, void* fu,
                                     void* fog, cudaStream_t s) const = 0;
    // the extraction's stencil gather: out[j] = sum_q w[q,j] u[index[q,j] + varoff]
    virtual cudaError_t gather(const void* u, int64_t varoff, int64_t npoints, int nper, const int64_t* index,
                               const void* w, void* out, cudaStream_t s) const = 0;
    // the regrid transfer of both variables, one new block per item
    virtual cudaError_t transfer(const TransferItem* items, int nitems, int E, const void* src, void* dst,
                                 cudaStream_t s) const = 0;
    virtual cudaError_t cf_ghosts(const CfFace* cf, int ncf, int E, const void* fu, const void* fog, void* ugd,
                                  void* gfd, void* ggd, cudaStream_t s) const = 0;
    // the coarse-fine image (I or R) of `vars` face planes per slot (vars, N^(D-1)) into dst
    virtual cudaError_t cf_planes(const CfFace* cf, int ncf, int E, const void* src, void* dst, int vars,
                                  cudaStream_t s) const = 0;
    virtual cudaError_t stage(const BlockItem* items, int nitems, int E, int mode, int truncate,
                              const StagePtrs& p, int grid, cudaStream_t s) const = 0;
    virtual cudaError_t energy(const BlockItem* items, int nitems, int E, const StagePtrs& p,
                               cudaStream_t s) const = 0;
    // coef: sqrt(g) at variable 0 of ncoef per node (NULL: flat)
    virtual cudaError_t norm(const BlockItem* items, int nitems, int E, const void* u, const void* ref, int p,
                             int vars_mask, double* num, double* vol, const void* coef, int ncoef,
                             cudaStream_t s) const = 0;
    virtual cudaError_t truncate(const BlockItem* items, int nitems, int E, void* u, const void* trm,
                                 const void* trd, cudaStream_t s) const = 0;
    // full metric (D = 3): mode 0 rhs, 1..4 RK stages, 5 energy; returns cudaErrorNotSupported for D != 3
    virtual cudaError_t fm_gradient(const BlockItem* items, int nitems, int E, int mode, const FmPtrs& p,
                                    cudaStream_t s) const = 0;
    virtual cudaError_t fm_stage(const BlockItem* items, int nitems, int E, int mode, int truncate,
                                 const FmPtrs& p, cudaStream_t s) const = 0;
    virtual cudaError_t fm_truncate(const BlockItem* items, int nitems, int E, const FmPtrs& p,
                                    cudaStream_t s) const = 0;
    virtual cudaError_t fm_energy(const BlockItem* items, int nitems, int E, const FmPtrs& p,
                                  cudaStream_t s) const = 0;
    virtual cudaError_t maxabs(const BlockItem* items, int nitems, int E, const void* u, int var, double* part,
                               cudaStream_t s) const = 0;
    // modes[0..nq): Legendre modes; weights/pows per mode; post factor; result tau (E^D per block)
    virtual cudaError_t modes(const BlockItem* items, int nitems, int E, const void* u, int var, int nq,
                              const int* modes, const double* weights, const double* pows, double post,
                              void* tau, cudaStream_t s) const = 0;
};

// Factories, one per dimension (separate translation units). Return
// nullptr when (prec, P) has no instantiation.
Ops* make_ops_d1(int prec, int P, const ElementTables<double>& t64, const ElementTables<float>& t32);
Ops* make_ops_d2(int prec, int P, const ElementTables<double>& t64, const ElementTables<float>& t32);
Ops* make_ops_d3(int prec, int P, const ElementTables<double>& t64, const ElementTables<float>& t32);

}  // namespace twoldg
