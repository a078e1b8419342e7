// Greedy k-lookahead selection of a binary lattice on the device:
// Lattice::select_experiments (src/core/lattice_api.cpp:116-168).
//
// The reference scores every candidate e against the experiments chosen
// before it by walking all states: state s falls in group g, bit i of g set
// when s is a subset of experiment i (set_group_index / is_up_set,
// lattice_api.cpp:28-44), and the score is sum_g |mass(g) - 1/2^m|.  That is
// O(2^n) per candidate and O(4^n) per step.
//
// Here the group masses come from one down-set transform
//   D(E) = sum over states s subset of E of post(s)
// in exact u64 fixed point, built once per call:
//   * the mass of "s subset of every experiment in J" is D(intersection of J),
//   * a group's mass follows by inclusion-exclusion (a superset Moebius
//     transform over the m experiment bits), exact in modular u64 because
//     every true group mass is a non-negative integer below 2^62,
//   * the score times 2^m * Z is sum_g |2^m mass(g) - Z| in u128, exact.
// One warp scores one candidate (2^m gathers of D, at most 32 per lane),
// the argmin keeps the lowest public (bit-reversed) index on ties, as the
// reference's ascending candidate loop with a strict < does.

#include <cuda_runtime.h>

#include <cstdint>

#include "provider_internal.h"

namespace bgt_gpu
{

namespace
{

constexpr int kDownsetTile = 2048; // u64 entries per CTA tile (16 KB)
constexpr int kDownsetThreads = 256;
constexpr int kScoreThreads = 256;
constexpr int kScoreWarps = kScoreThreads / 32;

using u64 = unsigned long long;
using u128 = unsigned __int128;

// q (FP64, or FP32 when fp32) -> floor(q * 2^scale).
__global__ void lookahead_fixed(const void *q, int fp32, u64 count, int scale, u64 *d)
{
	for (u64 i = blockIdx.x * static_cast<u64>(blockDim.x) + threadIdx.x; i < count;
		 i += static_cast<u64>(gridDim.x) * blockDim.x)
	{
		const double v = fp32 ? static_cast<double>(static_cast<const float *>(q)[i]) : static_cast<const double *>(q)[i];
		d[i] = static_cast<u64>(ldexp(v, scale));
	}
}

// In-place down-set sums over the bits [lo, lo + nb) of d (2^n entries):
// for each bit b of the range and every E with b set, d[E] += d[E - b].  A CTA
// holds 2^nb rows (the range's bits, stride 2^lo) by `cols` consecutive
// entries (cols = 1 for lo = 0, else min(32, 2^lo)), so loads and stores run
// along contiguous memory.
__global__ void __launch_bounds__(kDownsetThreads) downset_pass(u64 *d, int lo, int nb, int logc)
{
	__shared__ u64 tile[kDownsetTile];
	const int cols = 1 << logc;
	const int entries = cols << nb;
	const u64 chunks = (u64{1} << lo) >> logc;
	const u64 hi = blockIdx.x / chunks;
	const u64 chunk = blockIdx.x % chunks;
	const u64 base = (hi << (lo + nb)) + (chunk << logc);
	for (int t = threadIdx.x; t < entries; t += blockDim.x)
		tile[t] = d[base + (static_cast<u64>(t >> logc) << lo) + (t & (cols - 1))];
	for (int j = 0; j < nb; j++)
	{
		__syncthreads();
		for (int t = threadIdx.x; t < entries; t += blockDim.x)
			if (((t >> logc) >> j) & 1)
				tile[t] += tile[t - (cols << j)];
	}
	__syncthreads();
	for (int t = threadIdx.x; t < entries; t += blockDim.x)
		d[base + (static_cast<u64>(t >> logc) << lo) + (t & (cols - 1))] = tile[t];
}

__device__ __forceinline__ bool key_less(u64 ahi, u64 alo, unsigned int apub, u64 bhi, u64 blo, unsigned int bpub)
{
	if (ahi != bhi)
		return ahi < bhi;
	if (alo != blo)
		return alo < blo;
	return apub < bpub;
}

// Scores candidates e = 1 .. 2^n - 1 against the previous experiments
// (their 2^(m-1) intersection masks, masks[0] = every subject); each CTA
// writes its best (score hi, score lo, public index) to out[3 * blockIdx.x].
// R > 1 (m > 5): one candidate per warp, group index J = lane * R + r.
// R = 1 (m <= 5): 32 / 2^m candidates per warp, lane = slot * 2^m + J, so
// small lookaheads keep every lane busy.
template <int R>
__global__ void __launch_bounds__(kScoreThreads) lookahead_score(const u64 *__restrict__ d, int n, int m,
																  const unsigned int *__restrict__ masks, u64 *out)
{
	constexpr int kLogR = R == 1 ? 0 : R == 2 ? 1 : R == 4 ? 2 : R == 8 ? 3 : R == 16 ? 4 : 5;
	__shared__ u64 s_hi[kScoreThreads], s_lo[kScoreThreads];
	__shared__ unsigned int s_pub[kScoreThreads];
	const unsigned int lane = threadIdx.x & 31u;
	const unsigned int warp = threadIdx.x >> 5;
	const int groups = 1 << m;
	const int prev = m - 1;
	const int per_warp = R == 1 ? 32 / groups : 1; // candidates per warp
	const unsigned int slot = R == 1 ? lane >> m : 0u;
	const unsigned int jbase = R == 1 ? lane & static_cast<unsigned int>(groups - 1) : lane * R;
	const unsigned int full = n >= 32 ? 0xFFFFFFFFu : ((1u << n) - 1u);
	const u64 z = d[full];
	u64 best_hi = ~u64{0}, best_lo = ~u64{0};
	unsigned int best_pub = 0xFFFFFFFFu;
	const unsigned long long total = 1ull << n;
	const unsigned long long stride = static_cast<unsigned long long>(gridDim.x) * kScoreWarps * per_warp;
	for (unsigned long long c0 = (blockIdx.x * static_cast<unsigned long long>(kScoreWarps) + warp) * per_warp + 1;
		 c0 < total; c0 += stride)
	{
		const unsigned long long c = c0 + slot;
		const bool valid = c < total;
		const unsigned int e = static_cast<unsigned int>(c);
		u64 f[R];
#pragma unroll
		for (int r = 0; r < R; r++)
		{
			const unsigned int J = jbase + r;
			const unsigned int x = masks[J & ((1u << prev) - 1u)];
			f[r] = valid ? d[(J >> prev) & 1u ? (e & x) : x] : 0;
		}
		// Superset Moebius transform: mass(g) = sum_{J >= g} (-1)^{|J - g|} S(J).
#pragma unroll
		for (int b = 0; b < kLogR; b++)
		{
#pragma unroll
			for (int r = 0; r < R; r++)
				if (!((r >> b) & 1))
					f[r] -= f[r | (1 << b)];
		}
		for (int b = kLogR; b < m; b++)
		{
			const unsigned int lb = 1u << (b - kLogR);
#pragma unroll
			for (int r = 0; r < R; r++)
			{
				const u64 other = __shfl_xor_sync(0xFFFFFFFFu, f[r], lb);
				if (!(lane & lb))
					f[r] -= other;
			}
		}
		u128 acc = 0;
#pragma unroll
		for (int r = 0; r < R; r++)
		{
			const u128 scaled = static_cast<u128>(f[r]) << m;
			acc += scaled >= z ? scaled - z : static_cast<u128>(z) - scaled;
		}
		u64 lo = static_cast<u64>(acc), hi = static_cast<u64>(acc >> 64);
		// Sum over the lanes of one candidate: a segment of 2^m lanes (R = 1)
		// or the whole warp.
		const int span = R == 1 ? groups : 32;
		for (int off = span >> 1; off > 0; off >>= 1)
		{
			const u64 olo = __shfl_down_sync(0xFFFFFFFFu, lo, off);
			const u64 ohi = __shfl_down_sync(0xFFFFFFFFu, hi, off);
			const u64 sum = lo + olo;
			hi += ohi + (sum < lo ? 1u : 0u);
			lo = sum;
		}
		const unsigned int pub = __brev(e) >> (32 - n);
		if (valid && (lane & static_cast<unsigned int>(span - 1)) == 0 && key_less(hi, lo, pub, best_hi, best_lo, best_pub))
		{
			best_hi = hi;
			best_lo = lo;
			best_pub = pub;
		}
	}
	s_hi[threadIdx.x] = best_hi;
	s_lo[threadIdx.x] = best_lo;
	s_pub[threadIdx.x] = best_pub;
	for (int off = kScoreThreads / 2; off > 0; off >>= 1)
	{
		__syncthreads();
		if (static_cast<int>(threadIdx.x) < off)
		{
			const int o = threadIdx.x + off;
			if (key_less(s_hi[o], s_lo[o], s_pub[o], s_hi[threadIdx.x], s_lo[threadIdx.x], s_pub[threadIdx.x]))
			{
				s_hi[threadIdx.x] = s_hi[o];
				s_lo[threadIdx.x] = s_lo[o];
				s_pub[threadIdx.x] = s_pub[o];
			}
		}
	}
	if (threadIdx.x == 0)
	{
		out[3 * blockIdx.x] = s_hi[0];
		out[3 * blockIdx.x + 1] = s_lo[0];
		out[3 * blockIdx.x + 2] = s_pub[0];
	}
}

// The least of `blocks` CTA results; writes the winner's internal index.
__global__ void __launch_bounds__(256) lookahead_reduce(const u64 *in, int blocks, int n, unsigned int *result)
{
	__shared__ u64 s_hi[256], s_lo[256];
	__shared__ unsigned int s_pub[256];
	u64 bh = ~u64{0}, bl = ~u64{0};
	unsigned int bp = 0xFFFFFFFFu;
	for (int i = threadIdx.x; i < blocks; i += blockDim.x)
	{
		const u64 h = in[3 * i], l = in[3 * i + 1];
		const unsigned int p = static_cast<unsigned int>(in[3 * i + 2]);
		if (key_less(h, l, p, bh, bl, bp))
		{
			bh = h;
			bl = l;
			bp = p;
		}
	}
	s_hi[threadIdx.x] = bh;
	s_lo[threadIdx.x] = bl;
	s_pub[threadIdx.x] = bp;
	for (int off = 128; off > 0; off >>= 1)
	{
		__syncthreads();
		if (static_cast<int>(threadIdx.x) < off)
		{
			const int o = threadIdx.x + off;
			if (key_less(s_hi[o], s_lo[o], s_pub[o], s_hi[threadIdx.x], s_lo[threadIdx.x], s_pub[threadIdx.x]))
			{
				s_hi[threadIdx.x] = s_hi[o];
				s_lo[threadIdx.x] = s_lo[o];
				s_pub[threadIdx.x] = s_pub[o];
			}
		}
	}
	if (threadIdx.x == 0)
		*result = s_pub[0] == 0xFFFFFFFFu ? 0u : __brev(s_pub[0]) >> (32 - n);
}

} // namespace

int lookahead_score_blocks(int n)
{
	const unsigned long long warps = (1ull << n) - 1;
	const unsigned long long need = (warps + kScoreWarps - 1) / kScoreWarps;
	const unsigned long long cap = static_cast<unsigned long long>(sm_count()) * 8;
	return static_cast<int>(need < cap ? need : cap);
}

void launch_downset(const void *q, int fp32, int n, int scale, unsigned long long *d, cudaStream_t stream)
{
	const u64 count = u64{1} << n;
	const unsigned int fixed_blocks =
		static_cast<unsigned int>(count < 256ull * 1216 ? (count + 255) / 256 : 1216ull);
	lookahead_fixed<<<fixed_blocks, 256, 0, stream>>>(q, fp32, count, scale, d);
	cuda_check(cudaGetLastError(), "lookahead fixed-point launch");
	count_launches(1);
	int lo = 0;
	while (lo < n)
	{
		// Tiles of 2^nb rows x 2^logc columns, at most kDownsetTile entries.
		const int logc = lo == 0 ? 0 : (lo < 5 ? lo : 5);
		int nb = n - lo;
		const int cap = (lo == 0 ? 11 : 11 - logc);
		if (nb > cap)
			nb = cap;
		const u64 blocks = count >> (nb + logc);
		downset_pass<<<static_cast<unsigned int>(blocks), kDownsetThreads, 0, stream>>>(d, lo, nb, logc);
		cuda_check(cudaGetLastError(), "down-set pass launch");
		count_launches(1);
		lo += nb;
	}
}

void launch_lookahead_select(const unsigned long long *d, int n, int m, const unsigned int *masks,
							 unsigned long long *scratch, int blocks, unsigned int *result, cudaStream_t stream)
{
	const int groups = 1 << m;
	const int r = groups <= 32 ? 1 : groups / 32;
	switch (r)
	{
	case 1:
		lookahead_score<1><<<blocks, kScoreThreads, 0, stream>>>(d, n, m, masks, scratch);
		break;
	case 2:
		lookahead_score<2><<<blocks, kScoreThreads, 0, stream>>>(d, n, m, masks, scratch);
		break;
	case 4:
		lookahead_score<4><<<blocks, kScoreThreads, 0, stream>>>(d, n, m, masks, scratch);
		break;
	case 8:
		lookahead_score<8><<<blocks, kScoreThreads, 0, stream>>>(d, n, m, masks, scratch);
		break;
	case 16:
		lookahead_score<16><<<blocks, kScoreThreads, 0, stream>>>(d, n, m, masks, scratch);
		break;
	default:
		lookahead_score<32><<<blocks, kScoreThreads, 0, stream>>>(d, n, m, masks, scratch);
		break;
	}
	cuda_check(cudaGetLastError(), "lookahead score launch");
	lookahead_reduce<<<1, 256, 0, stream>>>(scratch, blocks, n, result);
	cuda_check(cudaGetLastError(), "lookahead reduce launch");
	count_launches(2);
}

} // namespace bgt_gpu
