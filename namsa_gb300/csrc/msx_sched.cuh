// Type-erased schedule table: for every compiled (line length, schedule) the
// launchers of the plain passes (msx_passes.cuh) and of the persistent
// TMA-pipelined passes (msx_tma.cuh).
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include "msx_passes.cuh"
#include "msx_tma.cuh"

namespace msx {

struct SchedOps {
  int n;                      // line length
  const char* name;
  int tw_words;
  int col_c;                  // columns per column-pass tile
  int col_boxr;               // rows per tensor-map box of the column tile
  void (*host_twiddles)(float2*);
  cudaError_t (*configure)();
  cudaError_t (*row)(float2* psi, const float2* trans, const float2* tw, int G, int Ny, cudaStream_t st);
  cudaError_t (*col)(int mode, const ColArgs& a, cudaStream_t st);
  // persistent passes; `ctas` = resident CTAs to launch (SMs x occupancy)
  cudaError_t (*row_tma)(const TmaPassArgs& a, int ctas, cudaStream_t st);
  cudaError_t (*col_tma)(const CUtensorMap& map, const TmaPassArgs& a, int ctas, cudaStream_t st);
  cudaError_t (*occupancy)(int* row_per_sm, int* col_per_sm);
  // row pass with a RowMode other than ROW_FULL (real-space stepping)
  cudaError_t (*row_mode)(int rmode, float2* psi, const float2* trans, const float2* tw, int G, int Ny, cudaStream_t st);
};

template <class S> struct SchedImpl {
  static void host_twiddles(float2* tw) { S::FFT::host_twiddles(tw); }
  static cudaError_t configure() {
    cudaError_t e = cudaFuncSetAttribute(row_pass_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)S::row_smem());
    const int cs = (int)S::col_smem();
    if (e == cudaSuccess) e = cudaFuncSetAttribute(col_pass_kernel<S, COL_INIT>, cudaFuncAttributeMaxDynamicSharedMemorySize, cs);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(col_pass_kernel<S, COL_MID>, cudaFuncAttributeMaxDynamicSharedMemorySize, cs);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(col_pass_kernel<S, COL_FINAL>, cudaFuncAttributeMaxDynamicSharedMemorySize, cs);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(col_pass_kernel<S, COL_INIT_FINAL>, cudaFuncAttributeMaxDynamicSharedMemorySize, cs);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(col_pass_kernel<S, COL_DETECT>, cudaFuncAttributeMaxDynamicSharedMemorySize, cs);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(row_pass_kernel<S, ROW_TF>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::row_smem());
    if (e == cudaSuccess) e = cudaFuncSetAttribute(row_pass_kernel<S, ROW_I>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::row_smem());
    if (e == cudaSuccess) e = cudaFuncSetAttribute(row_pass_kernel<S, ROW_F>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::row_smem());
    if (e == cudaSuccess) e = cudaFuncSetAttribute(row_pass_tma_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)RowTma<S>::smem());
    if (e == cudaSuccess) e = cudaFuncSetAttribute(col_mid_tma_kernel<S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ColTma<S>::smem());
    return e;
  }
  static cudaError_t row(float2* psi, const float2* trans, const float2* tw, int G, int Ny, cudaStream_t st) {
    const int lines = G * Ny;
    const int blocks = (lines + S::ROW_LINES - 1) / S::ROW_LINES;
    row_pass_kernel<S><<<blocks, S::THREADS, S::row_smem(), st>>>(psi, trans, tw, G, Ny);
    return cudaGetLastError();
  }
  static cudaError_t col(int mode, const ColArgs& a, cudaStream_t st) {
    const int tiles = (a.ncols + S::C - 1) / S::C;
    const dim3 grid(tiles * a.G);
    const size_t sm = S::col_smem();
    switch (mode) {
      case COL_INIT: col_pass_kernel<S, COL_INIT><<<grid, S::THREADS, sm, st>>>(a); break;
      case COL_MID: col_pass_kernel<S, COL_MID><<<grid, S::THREADS, sm, st>>>(a); break;
      case COL_FINAL: col_pass_kernel<S, COL_FINAL><<<grid, S::THREADS, sm, st>>>(a); break;
      case COL_DETECT: col_pass_kernel<S, COL_DETECT><<<grid, S::THREADS, sm, st>>>(a); break;
      default: col_pass_kernel<S, COL_INIT_FINAL><<<grid, S::THREADS, sm, st>>>(a); break;
    }
    return cudaGetLastError();
  }
  static cudaError_t row_tma(const TmaPassArgs& a, int ctas, cudaStream_t st) {
    const int ntiles = a.Ny * ((a.G + S::ROW_LINES - 1) / S::ROW_LINES);
    const int grid = ntiles < ctas ? ntiles : ctas;
    row_pass_tma_kernel<S><<<grid, S::THREADS, RowTma<S>::smem(), st>>>(a);
    return cudaGetLastError();
  }
  static cudaError_t col_tma(const CUtensorMap& map, const TmaPassArgs& a, int ctas, cudaStream_t st) {
    const int ntiles = ((a.x_hi > 0 ? a.x_hi : a.Nx) / S::C - a.x_lo / S::C) * a.G;
    if (ntiles <= 0) return cudaSuccess;
    const int grid = ntiles < ctas ? ntiles : ctas;
    col_mid_tma_kernel<S><<<grid, S::THREADS, ColTma<S>::smem(), st>>>(map, a);
    return cudaGetLastError();
  }
  static cudaError_t occupancy(int* row_per_sm, int* col_per_sm) {
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(row_per_sm, row_pass_tma_kernel<S>, S::THREADS,
                                                                  RowTma<S>::smem());
    if (e == cudaSuccess)
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(col_per_sm, col_mid_tma_kernel<S>, S::THREADS, ColTma<S>::smem());
    return e;
  }
  static cudaError_t row_mode(int rmode, float2* psi, const float2* trans, const float2* tw, int G, int Ny,
                              cudaStream_t st) {
    const int lines = G * Ny;
    const int blocks = (lines + S::ROW_LINES - 1) / S::ROW_LINES;
    switch (rmode) {
      case ROW_TF: row_pass_kernel<S, ROW_TF><<<blocks, S::THREADS, S::row_smem(), st>>>(psi, trans, tw, G, Ny); break;
      case ROW_I: row_pass_kernel<S, ROW_I><<<blocks, S::THREADS, S::row_smem(), st>>>(psi, trans, tw, G, Ny); break;
      case ROW_F: row_pass_kernel<S, ROW_F><<<blocks, S::THREADS, S::row_smem(), st>>>(psi, trans, tw, G, Ny); break;
      default: row_pass_kernel<S, ROW_FULL><<<blocks, S::THREADS, S::row_smem(), st>>>(psi, trans, tw, G, Ny); break;
    }
    return cudaGetLastError();
  }
  static SchedOps ops(const char* name) {
    return SchedOps{S::N, name, S::TW, S::C, ColTma<S>::BOXR, &host_twiddles, &configure, &row, &col,
                    &row_tma, &col_tma, &occupancy, &row_mode};
  }
};

// Schedules compiled for each line length (one translation unit per length).
int schedules_64(const SchedOps** out);
int schedules_128(const SchedOps** out);
int schedules_256(const SchedOps** out);
int schedules_384(const SchedOps** out);
int schedules_512(const SchedOps** out);
int schedules_768(const SchedOps** out);
int schedules_1024(const SchedOps** out);

}  // namespace msx
