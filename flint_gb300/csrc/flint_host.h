// flint_host.h -- internal host-side declarations shared by the .cu files.
#pragma once
#include <cstdint>
#include <string>
#include <cuda_runtime.h>
#include "flint_dev.cuh"
#include "../../include/flint_gpu.h"

namespace flint {

void count_launch();
cudaError_t probe_fp64(double* tflops);
cudaError_t launch_exp_selftest(const uint8_t* img, const ImageLayout& L, int64_t n, const double* x, double* y,
                                cudaStream_t st);
int device_sms();

cudaError_t launch_wdot(const uint8_t* img, const ImageLayout& L, int64_t n, int layout, const double* T,
                        const double* p, const double* Y, double* wdot, double* cp, double* h, cudaStream_t st);
cudaError_t launch_thermo(const uint8_t* img, const ImageLayout& L, int64_t n, int layout, const double* T,
                          const double* Y, double* cp, double* h, cudaStream_t st);
cudaError_t launch_chemistry_source(const uint8_t* img, const ImageLayout& L, int64_t n, double* roi,
                                    const double* T, double* omegadot, cudaStream_t st);
cudaError_t launch_wdot_jac(const uint8_t* img, const ImageLayout& L, int64_t n, int layout, const double* T,
                            const double* p, const double* Y, double* wdot, double* jac, cudaStream_t st);
cudaError_t launch_rhs(const uint8_t* img, const ImageLayout& L, int64_t n, const double* T, const double* p,
                       const double* Y, double* f, cudaStream_t st);
int reactor_slots(const ImageLayout& L);
size_t reactor_slot_bytes();
cudaError_t launch_reactor(const uint8_t* img, const ImageLayout& L, int64_t n, double* T, const double* p,
                           double* Y, const double* dt, const flint_reactor_opts& o, int* status, int* nsteps,
                           unsigned int* work_counter, double* jsave, int slots, cudaStream_t st);

size_t reactor_noalloc_bytes();
int reactor_noalloc_slots();
cudaError_t launch_reactor_noalloc(const uint8_t* img, const ImageLayout& L, int64_t n, double* T, const double* p,
                                   double* Y, const double* dt, const flint_reactor_opts& o, int* status,
                                   int* nsteps, cudaStream_t st);

// tabulated (reference general-loop) path, flint_table.cu
int table_create(const flint_table_desc* d, void** out, std::string& err);
void table_destroy(void* th);
int table_ns(void* th);
int table_nr(void* th);
cudaError_t table_run(void* th, int64_t n, int rhs, const double* roi, const double* T, double* out,
                      cudaStream_t st);

}  // namespace flint
