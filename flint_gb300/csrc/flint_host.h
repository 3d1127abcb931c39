// flint_host.h -- internal host-side declarations shared by the .cu files.
#pragma once
#include <cstdint>
#include <string>
#include <vector>
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include "flint_dev.cuh"
#include "../../include/flint_gpu.h"

// FLINT input files parsed on the host (flint_files.cu): the arrays of
// flint_table_desc, owned here, in its Fortran layout.
struct flint_table_set_s {
  int ns = 0, tmin = 0, tmax = 0, ti1 = 0, ti2 = 0;
  int nr[3] = {0, 0, 0};   // Arrhenius, Troe, Lindemann
  std::vector<std::string> names;
  std::vector<double> wm, cp, h, mu, kt;
  std::vector<double> ni1[3], ni2[3], eps[3];
  std::vector<double> kf, kb, ktroe[4], klind[3];
};

// A parsed mechanism IR blob (flint_ir.cu): the arrays of flint_mech_desc.
struct flint_ir_s {
  int ns = 0, nr = 0, flags = 0;
  double consts[3] = {0.0, 0.0, 0.0};   // r_eos, r_thermo, p_ref
  std::vector<double> mw, nasa7, arrh, arrh0, troe, rnu, rord, pnu, eff, nasa9;
  std::vector<int> rtype, reversible, rsp, psp;
};

namespace flint {

void count_launch();
cudaError_t probe_fp64(double* tflops);
cudaError_t launch_exp_selftest(const uint8_t* img, const ImageLayout& L, int64_t n, const double* x, double* y,
                                cudaStream_t st);
cudaError_t launch_log_selftest(const uint8_t* img, const ImageLayout& L, int64_t n, const double* x, double* y,
                                cudaStream_t st);
int device_sms();
// NVTX range over a scope of host code (the phase that enqueues a group of
// launches), so that a profiler can attribute kernels to phases; a no-op
// unless a tool is attached.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};
// Largest dynamic shared memory a block may opt into on the current device.
size_t device_smem_optin();
// Opt a kernel into `bytes` of dynamic shared memory.  A refusal is returned
// and consumed, so that it does not surface in a later cudaGetLastError.
inline cudaError_t set_smem(const void* fn, size_t bytes) {
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) (void)cudaGetLastError();
  return e;
}

// threads: threads per block of the warp kernels (64, 128 or 256; 0 = 256)
cudaError_t launch_wdot(const uint8_t* img, const ImageLayout& L, int64_t n, int layout, const double* T,
                        const double* p, const double* Y, double* wdot, double* cp, double* h, cudaStream_t st,
                        int threads = 0);
int warp_block_candidates(int* out);
bool use_small_kernel(const ImageLayout& L);   // wdot of <= 8 species: thread per cell
cudaError_t launch_species_thermo(const uint8_t* img, const ImageLayout& L, int64_t n, const double* T, double* cp,
                                  double* h, double* s, double* g, cudaStream_t st);
cudaError_t launch_thermo(const uint8_t* img, const ImageLayout& L, int64_t n, int layout, const double* T,
                          const double* Y, double* cp, double* h, cudaStream_t st);
cudaError_t launch_chemistry_source(const uint8_t* img, const ImageLayout& L, int64_t n, double* roi,
                                    const double* T, double* omegadot, cudaStream_t st);
cudaError_t launch_wdot_jac(const uint8_t* img, const ImageLayout& L, int64_t n, int layout, const double* T,
                            const double* p, const double* Y, double* wdot, double* jac, double* gscratch,
                            cudaStream_t st, int cv = 0, int threads = 0);   // cv: constant volume, p holds rho
int64_t warp_jac_scratch_doubles(const ImageLayout& L);
cudaError_t launch_rhs(const uint8_t* img, const ImageLayout& L, int64_t n, const double* T, const double* p,
                       const double* Y, double* f, cudaStream_t st, int cv = 0);
int reactor_slots(const ImageLayout& L);
size_t reactor_slot_bytes(const ImageLayout& L);
// Reactor layouts: the Newton matrix in shared memory (8 warps per block) or in
// the warp's global slot (8 or 4 warps per block).
enum { REACTOR_LAYOUT_AUTO = 0, REACTOR_LAYOUT_SHARED = 1, REACTOR_LAYOUT_GLOBAL = 2, REACTOR_LAYOUT_GLOBAL4 = 3,
       REACTOR_LAYOUT_GLOBAL2B = 4 };
// The layouts possible for this mechanism (what the autotuner chooses between); returns their count.
int reactor_layout_candidates(const ImageLayout& L, int* out);
cudaError_t launch_reactor(const uint8_t* img, const ImageLayout& L, int64_t n, double* T, const double* p,
                           double* Y, const double* dt, const flint_reactor_opts& o, int* status, int* nsteps,
                           unsigned int* work_counter, double* jsave, int slots, cudaStream_t st,
                           const unsigned long long* n_dev = nullptr,   // optional device-side cell count <= n
                           int layout = REACTOR_LAYOUT_AUTO);

size_t reactor_noalloc_bytes();
int reactor_noalloc_slots();
bool reactor_noalloc_fits(const ImageLayout& L);
cudaError_t launch_reactor_noalloc(const uint8_t* img, const ImageLayout& L, int64_t n, double* T, const double* p,
                                   double* Y, const double* dt, const flint_reactor_opts& o, int* status,
                                   int* nsteps, cudaStream_t st);

// learned surrogate, flint_surrogate.cu
struct Surrogate;
int surrogate_create(const uint8_t* mimg, const ImageLayout& L, unsigned int* counter, const flint_surrogate_desc* d,
                     Surrogate** out, std::string& err);
void surrogate_free(Surrogate* s);
int64_t surrogate_nparams(Surrogate* s);
int surrogate_features(Surrogate* s, int64_t n, const double* T, const double* p, const double* Y, const double* dt,
                       float* X, cudaStream_t st);
int surrogate_targets(Surrogate* s, int64_t n, const double* T0, const double* Y0, const double* T1, const double* Y1,
                      float* Yt, cudaStream_t st);
int surrogate_predict(Surrogate* s, int net, int64_t n, const float* X, float* Yn, cudaStream_t st);
int surrogate_train_step(Surrogate* s, int net, int64_t n, const float* X, const float* Yt, float lr, double* loss,
                         cudaStream_t st);
int surrogate_state(Surrogate* s, int net, float* host, int64_t* step, int get);
int surrogate_advance(Surrogate* s, int64_t n, double* T, const double* p, double* Y, const double* dt,
                      const flint_reactor_opts& o, const flint_surrogate_gate* gate, int* status, int* nsteps,
                      double* jsave, int jslots, double* metrics, bool want_counts, cudaStream_t st,
                      int reactor_layout = REACTOR_LAYOUT_AUTO);
void surrogate_counts(Surrogate* s, int64_t* acc, int64_t* rej);
int surrogate_set_forward(Surrogate* s, int mode);
int surrogate_forward_kind(Surrogate* s);
int surrogate_check(Surrogate* s, int* err);
int surrogate_read_counts(Surrogate* s, int64_t* acc, int64_t* rej);

// tabulated (reference general-loop) path, flint_table.cu
int table_create(const flint_table_desc* d, void** out, std::string& err);
void table_destroy(void* th);
int table_ns(void* th);
int table_nr(void* th);
cudaError_t table_run(void* th, int64_t n, int rhs, const double* roi, const double* T, double* out,
                      cudaStream_t st);
int table_has_transport(void* p);
cudaError_t table_transport(void* p, int64_t n, const double* rhoi, const double* T, double* mu, double* lam,
                            cudaStream_t st);
cudaError_t table_cons2prim(void* p, int64_t n, int np, const double* cons, const double* T, double* prim,
                            double* Tout, cudaStream_t st);

// FLINT's tabulated input files -> arrays (flint_files.cu)
int tables_read(const char* folder, const char* prefix, flint_table_set_s* t, std::string& err);
void tables_desc(const flint_table_set_s* t, flint_table_desc* d);

// mechanism IR blob -> arrays (flint_ir.cu)
int64_t ir_bytes(int ns, int nr, bool nasa9);
int ir_parse(const void* blob, int64_t bytes, flint_ir_s* ir, std::string& err);
void ir_desc(const flint_ir_s* ir, flint_mech_desc* d);

}  // namespace flint
