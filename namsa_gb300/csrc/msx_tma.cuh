// Persistent, TMA-pipelined versions of the two per-slice passes.
//
// Each CTA loops over tiles (a group of rows, or a group of columns of one
// wave).  While it transforms tile i out of one shared-memory stage, the bulk
// copy engine (cp.async.bulk for rows, cp.async.bulk.tensor for column tiles)
// fills the next stage(s) with the following tiles; one mbarrier per stage
// tracks the bytes in flight.  Row results go straight from registers to
// global memory; column results go back into their stage and out by a tiled
// bulk store.
//
// The row pass exchanges Stockham stages in place inside the staged rows, with
// an XOR swizzle of the element index (bits [S, S+4) folded into bits [0, 4))
// that keeps the per-stage scatters free of bank conflicts.  The column pass
// exchanges in the staged tile itself (columns interleaved element by
// element), and forms the propagator on the fly from separable factors:
//   P(kx, ky) mask(kx, ky) / N = px[kx] * py[ky]  for  lo[kx] <= ky <= hi[kx],  else 0,
// where [lo, hi] is the band of the float32 mask comparison in column kx.
//
// Waits: every mbarrier wait has a clock64 limit of about one second.  In the
// column pass thread 0 polls and publishes the outcome through shared memory
// and a CTA barrier, so the whole CTA leaves together; in the row pass each
// warp polls for itself and leaves on its own.  On a timeout the kernel sets
// bit 0 of *err, thread 0 waits (again bounded) for the copies it issued that
// have not landed, and the threads return.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include "msx_passes.cuh"

namespace msx {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: gives up after `limit` cycles (default 2^31, about one second at
// GB300 clocks).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, long long limit = (1LL << 31)) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity)) {
    if (clock64() - t0 > limit) return false;
  }
  return true;
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void tma2d_g2s(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

// Tiled bulk store of a shared-memory box to the tensor; completion is tracked
// by bulk groups of the issuing thread.
__device__ __forceinline__ void tma2d_s2g(const CUtensorMap* map, int x, int y, const void* src) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                   reinterpret_cast<uint64_t>(map)),
               "r"(x), "r"(y), "r"(smem_u32(src))
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// the issuing thread's bulk stores have read their shared memory
__device__ __forceinline__ void bulk_wait_read_all() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// the issuing thread's bulk stores are complete
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

// Row line inside a staged, densely packed row: element i lives at
// i ^ ((i >> SH) & 15).  SH = log2(elements per thread) makes the first
// Stockham scatter (stride E) and the gathers (stride T) conflict-free.
template <int SH>
struct SwizzledLine {
  float2* base;
  __host__ __device__ __forceinline__ float2& operator[](int i) const { return base[i ^ ((i >> SH) & 15)]; }
};

__host__ __device__ constexpr int ilog2(int v) { return v <= 1 ? 0 : 1 + ilog2(v / 2); }

struct TmaPassArgs {
  float2* psi;            // (Galloc, Ny, Nx) workspace
  const float2* trans;    // (Ny, Nx) transmission slice (row pass)
  const float2* tw;       // twiddles of the line schedule
  const float2* pyx;      // py[Ny] then px[Nx] (column pass)
  const int2* band;       // [lo, hi] ky band per column (column pass)
  int* err;               // bit 0: a bounded wait gave up; bit 1: misaligned shared memory
  int G, Ny, Nx;
  // columns [x_lo, x_hi) written by the row pass and processed by the column
  // pass (x_hi == 0: all); the columns outside hold zeros that stay zero
  int x_lo, x_hi;
};

// ----------------------------------------------------------------------------- row pass
// A tile is ROW_LINES rows of one y (from consecutive waves) plus that y's
// transmission row.  STAGES stages cycle through the CTA's tiles; thread 0 is
// the producer.  There is no CTA-wide barrier in the loop: every warp waits on
// the stage's `full` barrier itself, transforms its own rows in place, and
// releases the stage on its `empty` barrier (one arrival per warp) after a
// proxy fence (its in-place exchanges are generic-proxy writes that the next
// bulk copy into the stage must follow).  Thread 0 refills a stage only after
// all warps released it, so warps may drift up to STAGES - 1 tiles apart.
template <class S>
struct RowTma {
  static constexpr int NX = S::N;
  static constexpr int L = S::ROW_LINES;
  static constexpr int STAGE = (L + 1) * NX;  // float2 words: L rows + the transmission row
  static constexpr size_t bytes(int stages) {
    return sizeof(float2) * ((size_t)stages * STAGE + S::TW_PAD) + 2 * stages * sizeof(uint64_t);
  }
  // CTAs per SM that the shared memory allows (228 KB per SM, 1 KB reserved per CTA)
  static constexpr int fit(int stages) { return (int)(233472 / (bytes(stages) + 1024)); }
  // three stages when that keeps the occupancy the registers allow, else two
  static constexpr int STAGES = fit(3) >= (fit(2) < S::MINB ? fit(2) : S::MINB) ? 3 : 2;
  static constexpr size_t smem() { return bytes(STAGES); }
};

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

template <class S>
__global__ void __launch_bounds__(S::THREADS, S::MINB) row_pass_tma_kernel(TmaPassArgs a) {
  constexpr int NX = S::N, T = S::T, E = S::E, L = S::ROW_LINES, STAGE = RowTma<S>::STAGE;
  constexpr int NS = RowTma<S>::STAGES, WARPS = S::WARPS;
  extern __shared__ __align__(1024) float2 smem[];
  float2* stage = smem;
  float2* tw = smem + NS * STAGE;
  uint64_t* full = reinterpret_cast<uint64_t*>(tw + S::TW_PAD);
  uint64_t* empty = full + NS;
  const int tid = threadIdx.x;
  if constexpr (S::PAIRED) {  // the paired exchange addresses need 256-byte-aligned lines
    if (smem_u32(smem) & 255u) {
      if (tid == 0) atomicOr(a.err, 2);
      return;
    }
  }
  for (int i = tid; i < S::TW; i += blockDim.x) tw[i] = a.tw[i];
  if (tid == 0) {
    for (int s = 0; s < NS; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], WARPS);
    }
    fence_mbar_init();
  }
  __syncthreads();
  const int pchunks = (a.G + L - 1) / L;
  const int ntiles = a.Ny * pchunks;
  const int mine = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;

  auto issue = [&](int k) {  // this CTA's k-th tile into stage k % NS
    const int tile = blockIdx.x + k * gridDim.x;
    const int y = tile / pchunks, pc = tile - y * pchunks;
    const int p0 = pc * L;
    const int nl = min(L, a.G - p0);
    float2* dst = stage + (k % NS) * STAGE;
    uint64_t* bar = &full[k % NS];
    mbar_expect_tx(bar, (uint32_t)((nl + 1) * NX * sizeof(float2)));
    for (int i = 0; i < nl; ++i)
      bulk_g2s(dst + i * NX, a.psi + ((size_t)(p0 + i) * a.Ny + y) * NX, NX * sizeof(float2), bar);
    bulk_g2s(dst + L * NX, a.trans + (size_t)y * NX, NX * sizeof(float2), bar);
  };

  const int warp = tid >> 5, lane = tid & 31;
  const int lw = lane / T, t = lane % T;
  const int slot = warp * S::LPW + lw;  // line slot within a tile
  int issued = 0;                       // tiles handed to the copy engine (thread 0 only)
  if (tid == 0)
    for (; issued < NS - 1 && issued < mine; ++issued) issue(issued);
  for (int k = 0; k < mine; ++k) {
    const int s = k % NS;
    int pok = 1;
    if (warp == 0) {
      if (lane == 0 && issued < mine) {
        // the stage of tile `issued` last held tile issued - NS
        if (issued >= NS) pok = mbar_wait_bounded(&empty[issued % NS], ((issued / NS) - 1) & 1) ? 1 : 0;
        if (pok) issue(issued++);
      }
      pok = __shfl_sync(0xffffffffu, pok, 0);
    }
    const int ok = __all_sync(0xffffffffu, mbar_wait_bounded(&full[s], (k / NS) & 1) ? 1 : 0) && pok;
    if (!ok) {
      if (lane == 0) atomicOr(a.err, 1);
      if (tid == 0)  // copies in flight must land before the CTA's shared memory is released
        for (int j = k; j < issued; ++j) mbar_wait_bounded(&full[j % NS], (j / NS) & 1);
      return;
    }
    const int tile = blockIdx.x + k * gridDim.x;
    const int y = tile / pchunks, pc = tile - y * pchunks;
    const int p0 = pc * L;
    const int nl = min(L, a.G - p0);
    float2* line = stage + s * STAGE + slot * NX;
    const float2* trow = stage + s * STAGE + L * NX;
    float2 v[E];
#pragma unroll
    for (int m = 0; m < E; ++m) v[m] = line[t + T * m];
    if constexpr (S::PAIRED) {
      const unsigned la = smem_u32(line);
      PairedFFT512::run<true>(v, la, tw, t);
#pragma unroll
      for (int m = 0; m < E; ++m) v[m] = cmul(v[m], trow[t + T * m]);
      PairedFFT512::run<false>(v, la, tw, t);
    } else {
      SwizzledLine<ilog2(E)> buf{line};
      S::FFT::template run<true, false>(v, buf, tw, t);
#pragma unroll
      for (int m = 0; m < E; ++m) v[m] = cmul(v[m], trow[t + T * m]);
      S::FFT::template run<false, false>(v, buf, tw, t);
    }
    if (slot < nl) {
      float2* out = a.psi + ((size_t)(p0 + slot) * a.Ny + y) * NX;
      const int xlo = a.x_lo, xhi = a.x_hi > 0 ? a.x_hi : NX;
#pragma unroll
      for (int m = 0; m < E; ++m) {
        const int xk = t + T * m;
        if (xk >= xlo && xk < xhi) out[xk] = v[m];
      }
    }
    fence_proxy_async();  // this warp's exchanges precede the next bulk copy into the stage
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty[s]);
  }
}

// ----------------------------------------------------------------------------- column pass
// A tile is C columns of one wave (tensor-map boxes of BOXR rows x C columns,
// columns interleaved element by element).  The C columns' T threads each are
// spread over the CTA (thread = c + C t keeps every shared-memory access on
// consecutive columns), so exchanges use CTA barriers: #0, where every thread
// has waited for the tile's bytes (the outcome is combined with
// __syncthreads_and, so the CTA leaves together on a timeout) and has finished
// the previous tile, and then one after each exchange's scatter.  The
// exchanges alternate between a separate scratch and the tile's own stage
// (scratch first; the inverse transform continues the alternation), so no
// scatter needs a barrier before it: #0 orders the scratch against the previous
// tile's reads, the first exchange's barrier orders the stage against this
// tile's loads, and each later scatter is two exchanges after the last reads of
// its buffer.  Two-stage transforms take three barriers per tile, three-stage
// ones five.
// Where a third tile-sized buffer does not fit beside the two stages without
// costing occupancy, both transforms exchange in the stage and each scatter is
// preceded by a barrier as well.
// Results: every thread writes its outputs back into the tile's stage, at the
// words its own final gather read (so no barrier is needed before), and fences
// them for the async proxy; after the next tile's #0, thread 0 issues the
// tiled bulk store of the tile.  Thread 0 refills that stage with tile k+1
// after the forward transform of tile k (past #1), once the store has read
// the stage; after the last tile the CTA synchronises, stores it and waits
// for the store to complete.
// Order of a column pass's tiles: tile u of G waves x tiles_x column tiles
// starting at xt0 -> (wave p, column tile xt).  The tiles xt = 2j and 2j + 1 of
// one wave share the tensor map's 256-byte L2 fills, so they are taken one
// after the other (by neighbouring CTAs); a tile whose partner lies outside the
// range (at most one at each end) is ordered on its own.
__host__ __device__ __forceinline__ void col_tile_order(int u, int G, int xt0, int tiles_x, int& p, int& xt) {
  const int lead = xt0 & 1, npairs = (tiles_x - lead) >> 1;
  if (u < lead * G) {
    p = u; xt = xt0;
    return;
  }
  u -= lead * G;
  if (u < npairs * 2 * G) {
    const int q = u / (2 * G), r = u - q * 2 * G;
    p = r >> 1; xt = xt0 + lead + 2 * q + (r & 1);
    return;
  }
  p = u - npairs * 2 * G; xt = xt0 + tiles_x - 1;
}

template <class S>
struct ColTma {
  static constexpr int NY = S::N;
  static constexpr int C = S::C;
  static constexpr int BOXR = NY < 128 ? NY : 128;  // rows per tensor-map box
  static constexpr int NBOX = NY / BOXR;
  static constexpr int STAGE = C * NY;
  static constexpr size_t bytes(int buffers) { return 16 + sizeof(float2) * ((size_t)buffers * STAGE + S::TW_PAD + NY); }
  static constexpr int fit(int buffers) {
    return bytes(buffers) > 232448 ? 0 : (int)(233472 / (bytes(buffers) + 1024));
  }
  // a separate exchange scratch when it fits without costing occupancy; otherwise
  // both transforms exchange in the stage itself (two more barriers per tile)
  static constexpr bool SCRATCH = fit(3) >= (fit(2) < S::MINB ? fit(2) : S::MINB);
  static constexpr size_t smem() { return bytes(SCRATCH ? 3 : 2); }
};

template <class S>
__global__ void __launch_bounds__(S::THREADS, S::MINB) col_mid_tma_kernel(const __grid_constant__ CUtensorMap map,
                                                                        TmaPassArgs a) {
  constexpr int NY = S::N, T = S::T, E = S::E, C = S::C;
  constexpr int BOXR = ColTma<S>::BOXR, NBOX = ColTma<S>::NBOX, STAGE = ColTma<S>::STAGE;
  extern __shared__ __align__(1024) float2 smem[];
  constexpr bool SCR = ColTma<S>::SCRATCH;
  float2* stage = smem;
  float2* scratch = smem + 2 * STAGE;  // used when SCR
  float2* tw = stage + (SCR ? 3 : 2) * STAGE;
  float2* py = tw + S::TW_PAD;
  uint64_t* full = reinterpret_cast<uint64_t*>(py + NY);
  const int tid = threadIdx.x;
  for (int i = tid; i < S::TW; i += blockDim.x) tw[i] = a.tw[i];
  for (int i = tid; i < NY; i += blockDim.x) py[i] = a.pyx[i];
  if (tid == 0) {
    mbar_init(&full[0], 1);
    mbar_init(&full[1], 1);
    fence_mbar_init();
  }
  __syncthreads();
  const int xt0 = a.x_lo / C;  // column tiles xt0 .. xt0 + tiles_x - 1
  const int tiles_x = (a.x_hi > 0 ? a.x_hi : a.Nx) / C - xt0;
  const int ntiles = tiles_x * a.G;
  const int mine = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
  auto coords = [&](int u, int& p, int& xt) { col_tile_order(u, a.G, xt0, tiles_x, p, xt); };

  auto load = [&](int k) {  // this CTA's k-th tile into stage k & 1
    int p, xt;
    coords(blockIdx.x + k * gridDim.x, p, xt);
    float2* dst = stage + (k & 1) * STAGE;
    uint64_t* bar = &full[k & 1];
    mbar_expect_tx(bar, (uint32_t)(STAGE * sizeof(float2)));
#pragma unroll
    for (int b = 0; b < NBOX; ++b) tma2d_g2s(dst + b * BOXR * C, &map, xt * C, p * NY + b * BOXR, bar);
  };
  auto store = [&](int k) {  // the k-th tile's results, staged in stage k & 1, back to the workspace
    int p, xt;
    coords(blockIdx.x + k * gridDim.x, p, xt);
    const float2* src = stage + (k & 1) * STAGE;
#pragma unroll
    for (int b = 0; b < NBOX; ++b) tma2d_s2g(&map, xt * C, p * NY + b * BOXR, src + b * BOXR * C);
    bulk_commit();
  };

  const int c = tid % C, t = tid / C;
  int loaded = 0;  // tiles handed to the copy engine (thread 0 only)
  if (tid == 0)
    for (; loaded < 2 && loaded < mine; ++loaded) load(loaded);
  // this column's propagator factor and mask band, fetched one tile ahead
  auto column_of = [&](int k) {
    int p, xt;
    coords(blockIdx.x + k * gridDim.x, p, xt);
    return xt * C + c;
  };
  float2 px_next = make_float2(0.f, 0.f);
  int2 bd_next = make_int2(1, 0);
  if (mine > 0) {
    px_next = __ldg(a.pyx + NY + column_of(0));
    bd_next = __ldg(a.band + column_of(0));
  }
  for (int k = 0; k < mine; ++k) {
    const int s = k & 1;
    const float2 px = px_next;
    const int2 bd = bd_next;
    if (k + 1 < mine) {
      px_next = __ldg(a.pyx + NY + column_of(k + 1));
      bd_next = __ldg(a.band + column_of(k + 1));
    }
    const bool ok = mbar_wait_bounded(&full[s], (k >> 1) & 1);
    if (!__syncthreads_and(ok)) {  // #0
      if (tid == 0) {
        atomicOr(a.err, 1);
        bulk_wait_all();  // stores in flight read the stages
        for (int j = k; j < loaded; ++j) mbar_wait_bounded(&full[j & 1], (j >> 1) & 1);
      }
      return;
    }
    if (tid == 0 && k >= 1) store(k - 1);  // written back into its stage and fenced before #0
    float2* st = stage + s * STAGE;
    InterleavedLine<C> in{st + c};
    float2 v[E];
#pragma unroll
    for (int m = 0; m < E; ++m) v[m] = in[t + T * m];
    // with the scratch, the exchanges alternate scratch, stage, scratch, ... over
    // the forward transform and continue the alternation into the inverse one
    constexpr int NXCH = S::FFT::kExchanges;
    const InterleavedLine<C> scr{scratch + c};
    if constexpr (SCR)
      S::FFT::template run_alt<false, true, 0>(v, scr, in, tw, t);  // #1 (and one per further exchange)
    else
      S::FFT::template run<false, true, InterleavedLine<C>, true>(v, in, tw, t);
    if (tid == 0 && k >= 1 && loaded < mine) {  // tile k+1 into the stage of tile k-1, once its store has read it
      bulk_wait_read_all();
      load(loaded++);
    }
#pragma unroll
    for (int m = 0; m < E; ++m) {
      const int ky = t + T * m;
      const float2 f = (ky >= bd.x && ky <= bd.y) ? cmul(px, py[ky]) : make_float2(0.f, 0.f);
      v[m] = cmul(v[m], f);
    }
    if constexpr (SCR)
      S::FFT::template run_alt<true, true, NXCH % 2>(v, scr, in, tw, t);  // #2 ...
    else
      S::FFT::template run<true, true, InterleavedLine<C>, true>(v, in, tw, t);
    // results back into the stage, at the words this thread read last (the final
    // gather is from the stage), for the bulk store issued after the next #0
#pragma unroll
    for (int m = 0; m < E; ++m) in[t + T * m] = v[m];
    fence_proxy_async();  // these writes precede the bulk store and the refill of the stage
  }
  __syncthreads();
  if (tid == 0 && mine > 0) {
    store(mine - 1);
    bulk_wait_all();
  }
}

}  // namespace msx
