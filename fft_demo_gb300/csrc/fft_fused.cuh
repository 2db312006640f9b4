// Fused four-step transform: both passes of a large 1D FFT in one persistent
// launch, chunked so the intermediate stays in L2.
//
// N = N1 * N2. Pass 1 (length N1 down the columns of [N1][N2], outer twiddle
// W_N^{n2 k1}) writes a chunk of sequences into a workspace slot; pass 2
// (length N2 along the rows, transposing store) reads the slot and writes the
// output. Work items are handed out by one global atomic counter in the order
//   P1(0), P1(1), P2(0), P1(2), P2(1), ..., P2(nchunks-1)
// (each Pk(c) = all tiles of pass k for chunk c). Dependencies:
//   a P2(c) tile waits until every P1(c) tile is done;
//   a P1(c) tile with c >= ring waits until every P2(c - ring) tile is done
//   (its workspace slot is reused; ring >= 2).
// Items are taken in order, so every wait is for items already taken by
// running CTAs: no cycle can form. Waits are bounded (the error word is set
// and the item skipped if one gives up). The workspace ring (ring chunks of
// about 16 MiB) is rewritten while resident in L2, so HBM sees roughly one
// read of the input and one write of the output.
//
// In-place transforms are safe: chunk c's input is fully read by its P1
// tiles before any P2(c) tile writes chunk c's output. Pass 1 reads the input
// with non-coherent (ld.global.nc) loads even then: every address of `in` is
// read only by the P1 tiles of its own chunk, all of which finish (and are
// counted in done1) before the first P2 tile of that chunk writes it, and it
// is never read again in the launch; chunks start on sequence boundaries
// (multiples of 2^15 * 4 bytes), so no cache line holds two chunks. No load
// can therefore see a line that was written during the launch.
#pragma once
#include "fft_io.cuh"
#include "fft_tile.cuh"

namespace tcfft {

struct FusedSched {
  unsigned int* counter;  // next item
  int* done1;             // per chunk: pass-1 tiles finished
  int* done2;             // per chunk: pass-2 tiles finished
  int nchunks;
  int tiles1, tiles2;     // tiles per chunk
  int ring;               // workspace slots
  int chunk_seqs;         // sequences per chunk
  long long batch;        // sequences in total
  long long n;            // points per sequence
  unsigned int wait_polls;  // bound of each dependency wait (tcfft_set_wait_limit)
};

__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Spin (thread 0) until *p >= target; false if max_polls polls passed
// without it (max_polls = 0 gives up at once).
__device__ __forceinline__ bool wait_counter(const int* p, int target, uint32_t max_polls) {
  for (uint32_t i = 0; i < max_polls; ++i) {
    if (ld_acquire(p) >= target) return true;
    __nanosleep(i < 64 ? 32 : 256);
  }
  return false;
}

template <int L1, int G1, int L2, int G2, int SIGN>
__global__ void __launch_bounds__(kPassThreads, 2)
    fft_fourstep_fused(const IoHalf<false, false> io1_base, const IoHalf<true, false, true> io2_base,
                       const PassCore core1, const PassCore core2, const FusedSched sc) {
  constexpr uint32_t C1 = pass_tmem_cols<L1, G1>(), C2 = pass_tmem_cols<L2, G2>();
  constexpr uint32_t TMEM_COLS = C1 > C2 ? C1 : C2;
  __shared__ unsigned int s_item;
  __shared__ int s_ok;
  PassState st;
  pass_setup<TMEM_COLS>(st, core1.bmat);
  const unsigned int total = static_cast<unsigned int>(sc.nchunks) * (sc.tiles1 + sc.tiles2);
  const long long chunk_elems = static_cast<long long>(sc.chunk_seqs) * sc.n;
  bool alive = true;
  while (alive) {
    if (threadIdx.x == 0) s_item = atomicAdd(sc.counter, 1u);
    __syncthreads();
    const unsigned int item = s_item;
    if (item >= total) break;
    // decode: step 0 = P1(0); step r (1..nchunks-1) = P1(r) then P2(r-1); last = P2(nchunks-1)
    int pass, chunk, t;
    if (item < static_cast<unsigned int>(sc.tiles1)) {
      pass = 1;
      chunk = 0;
      t = static_cast<int>(item);
    } else {
      const unsigned int rest = item - sc.tiles1;
      const unsigned int per = sc.tiles1 + sc.tiles2;
      const int r = 1 + static_cast<int>(rest / per);
      const int k = static_cast<int>(rest % per);
      if (r < sc.nchunks && k < sc.tiles1) {
        pass = 1;
        chunk = r;
        t = k;
      } else {
        pass = 2;
        chunk = r - 1;
        t = r < sc.nchunks ? k - sc.tiles1 : k;
      }
    }
    const long long seq0 = static_cast<long long>(chunk) * sc.chunk_seqs;
    const long long nseq = (sc.batch - seq0) < sc.chunk_seqs ? (sc.batch - seq0) : sc.chunk_seqs;
    const int slot = chunk % sc.ring;
    // dependencies (thread 0 waits, the CTA follows)
    if (threadIdx.x == 0) {
      bool ok = true;
      if (pass == 2) ok = wait_counter(sc.done1 + chunk, sc.tiles1, sc.wait_polls);
      else if (chunk >= sc.ring) ok = wait_counter(sc.done2 + (chunk - sc.ring), sc.tiles2, sc.wait_polls);
      if (!ok) atomicOr(core1.err, kErrQueueTimeout);
      s_ok = ok;
    }
    __syncthreads();
    if (s_ok) {
      if (pass == 1) {
        IoHalf<false, false> io = io1_base;
        io.in = io1_base.in + seq0 * sc.n;
        io.out = io1_base.out + static_cast<long long>(slot) * chunk_elems;
        io.total_lines = nseq * (sc.n / L1);
        alive = pass_tile<L1, G1, true, SIGN>(st, io, core1, static_cast<long long>(t) * G1);
      } else {
        IoHalf<true, false, true> io = io2_base;
        io.in = io2_base.in + static_cast<long long>(slot) * chunk_elems;
        io.out = io2_base.out + seq0 * sc.n;
        io.total_lines = nseq * (sc.n / L2);
        alive = pass_tile<L2, G2, true, SIGN>(st, io, core2, static_cast<long long>(t) * G2);
      }
    }
    // publish: every thread's stores are visible device-wide before the count
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(pass == 1 ? sc.done1 + chunk : sc.done2 + chunk, 1);
  }
  pass_teardown<TMEM_COLS>(st);
}

template <int L1, int G1, int L2, int G2>
constexpr int fused_smem_bytes() {
  return pass_smem_bytes<L1, G1>() > pass_smem_bytes<L2, G2>() ? pass_smem_bytes<L1, G1>()
                                                                : pass_smem_bytes<L2, G2>();
}

}  // namespace tcfft
