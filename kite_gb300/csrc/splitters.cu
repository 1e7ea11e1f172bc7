// Tile splitters over the key space.  Splitters never change which .kite
// partition a key lands in (that is the Fibonacci hash); they only cut each
// hash bucket into key ranges small enough for the on-chip sort.
//
// Sampled-histogram splitters: a 2^16-bin histogram of the top key bits of
// sampled keys, cut at equal cumulative mass.  The learned alternative lives
// in mlp_kernels.cu and produces splitters in the same format.
#include "kite_internal.h"
#include "splitters.h"

namespace kite {

template <class T>
__global__ void k_sample_hist(const T* __restrict__ sample, uint32_t n, uint32_t key_bits, uint32_t hbits,
                              unsigned* __restrict__ hist) {
  const uint32_t sh = key_bits - hbits;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const uint32_t bin = (uint32_t)(uint64_t)(sample[i] >> sh);
    atomicAdd(&hist[bin], 1u);
  }
}

// One CTA: turns the histogram into its inclusive cumulative counts (in
// place), then splitter j = upper edge of the first bin whose cumulative
// count reaches ceil(j*total/S).
template <class T>
__global__ void __launch_bounds__(1024) k_hist_splitters(unsigned* __restrict__ cum, uint32_t hbits,
                                                         uint32_t key_bits, uint32_t S, T* __restrict__ spl) {
  __shared__ unsigned sm[34];
  const uint32_t nb = 1u << hbits;
  unsigned carry = 0;
  for (uint32_t b0 = 0; b0 < nb; b0 += 1024) {
    const uint32_t b = b0 + threadIdx.x;
    const unsigned v = b < nb ? cum[b] : 0;
    unsigned tot;
    const unsigned ex = block_exclusive_scan<1024, unsigned>(v, sm, &tot);
    if (b < nb) cum[b] = carry + ex + v;
    carry += tot;
  }
  __syncthreads();
  const unsigned long long total = carry;
  const uint32_t sh = key_bits - hbits;
  for (uint32_t j = threadIdx.x + 1; j < S; j += blockDim.x) {
    T s;
    if (total == 0) {
      // no sample: uniform cut of [0, 2^key_bits): j/S as a 32-bit fraction, scaled
      const unsigned long long f = ((unsigned long long)j << 32) / S;
      s = key_bits >= 32 ? ((T)f << (key_bits - 32)) : (T)(f >> (32 - key_bits));
    } else {
      const unsigned long long target = (total * (unsigned long long)j + S - 1) / S;
      uint32_t lo = 0, hi = nb - 1;
      while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if ((unsigned long long)cum[mid] >= target) hi = mid;
        else lo = mid + 1;
      }
      // keys of bins <= lo fall below the splitter
      s = (lo + 1 == nb && key_bits == (uint32_t)KeyTraits<T>::kBits) ? ~T(0) : ((T)(lo + 1) << sh);
    }
    spl[j - 1] = s;
  }
}

template <class T>
int compute_hist_splitters(const T* d_sample, uint32_t nsample, uint32_t key_bits, uint32_t S, T* d_spl,
                           unsigned* d_hist /* 65536 */, cudaStream_t s) {
  const uint32_t hbits = key_bits < 16 ? key_bits : 16;
  cudaMemsetAsync(d_hist, 0, sizeof(unsigned) << hbits, s);
  if (nsample) k_sample_hist<T><<<256, 256, 0, s>>>(d_sample, nsample, key_bits, hbits, d_hist);
  k_hist_splitters<T><<<1, 1024, 0, s>>>(d_hist, hbits, key_bits, S, d_spl);
  return nsample ? 2 : 1;
}
template int compute_hist_splitters<uint64_t>(const uint64_t*, uint32_t, uint32_t, uint32_t, uint64_t*, unsigned*,
                                              cudaStream_t);
template int compute_hist_splitters<u128>(const u128*, uint32_t, uint32_t, uint32_t, u128*, unsigned*,
                                          cudaStream_t);

}  // namespace kite
