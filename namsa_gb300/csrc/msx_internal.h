// Internal declarations shared by the translation units of libmsx.so.
#pragma once
#include <cuda_runtime.h>

#include "msx_sched.cuh"

namespace msx {

cudaError_t launch_atom_windows(const double* coeff, int nspecies, int n0, int n1, int os, double range, float* out,
                                cudaStream_t st);
cudaError_t launch_potential(const int4* sites, const int* slice_off, int num_slices, const float* windows, int H, int W,
                             int Ny, int Nx, float sigma, float2* trans, float* pot, cudaStream_t st);
cudaError_t launch_probe(int Ny, int Nx, float kmax, double lambda, float k_semi, double C1, double C3, double C5,
                         int smooth, float2* psik, float* aperture, double* norm, cudaStream_t st);
// *dst = value, as a one-thread kernel on st.
cudaError_t launch_store_double(double* dst, double value, cudaStream_t st);
// Sets the message returned by msx_last_error for the calling thread.
void set_last_error(const char* msg);

cudaError_t launch_detect_reduce(const float* partial, int G, int tiles, int ndet, float* out, cudaStream_t st);
cudaError_t launch_pfac(int Ny, int Nx, float kmax, double lambda, double slice_t, float k_band, float2* pyx,
                        int2* band, cudaStream_t st);
cudaError_t launch_ptab(int Ny, int Nx, float kmax, double lambda, double slice_t, float k_band, float2* ptab,
                        cudaStream_t st);

}  // namespace msx
