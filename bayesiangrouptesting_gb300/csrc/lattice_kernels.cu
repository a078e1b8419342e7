// Kernels of the GB300 lattice provider (see lattice_kernels.cuh for the
// design).  All kernels index the lattice they work on through
// states[blockIdx.y], so one launch can sweep many same-shape lattices (all
// tree nodes of one depth, or a batch of sessions).
#include <cuda_runtime.h>

#include "lattice_kernels.cuh"

namespace bgt_gpu
{

// ------------------------------------------------------------------ K1

// Classification of one atom from its fixed-point mass (update_metadata,
// src/core/model/lattice_base.cpp:246-264): mass < lo -> positive,
// mass > 1 - up -> negative, classified atoms are never revisited.
__device__ __forceinline__ void classify_atoms(LatticeDev &L, double up, double lo)
{
	const double zg = __ull2double_rn(L.z_g);
	unsigned int pos = L.pos, neg = L.neg;
	for (int i = 0; i < L.atoms; i++)
	{
		const unsigned int bit = 1u << i;
		if ((pos | neg) & bit)
			continue;
		const double m = __ull2double_rn(__ldcg(L.atom_fixed + i)) / zg;
		if (m < lo)
			pos |= bit;
		else if (m > (1 - up))
			neg |= bit;
	}
	L.pos = pos;
	L.neg = neg;
}


// Block-wide float sum over 1024 threads; result valid in every thread.
__device__ __forceinline__ float block_sum_1024(float v, float *red)
{
	for (int o = 16; o > 0; o >>= 1)
		v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
	const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
	if (lane == 0)
		red[warp] = v;
	__syncthreads();
	float t = lane < (kTileThreads / 32) ? red[lane] : 0.0f;
	for (int o = 16; o > 0; o >>= 1)
		t += __shfl_xor_sync(0xFFFFFFFFu, t, o);
	return t;
}

// In-register zeta over the 4 bits of the per-thread index i, for those of
// the lattice bits `bit0 .. bit0+3` that lie below `tbits`.
__device__ __forceinline__ void reg_zeta16(unsigned long long (&a)[kPerThread], int bit0, int tbits)
{
#pragma unroll
	for (int lvl = 0; lvl < 4; lvl++)
	{
		if (bit0 + lvl < tbits)
		{
#pragma unroll
			for (int i = 0; i < kPerThread; i++)
				if (!(i & (1 << lvl)))
					a[i] += a[i | (1 << lvl)];
		}
	}
}

// One K1 tile: see the header.  Dynamic shared memory: 2^14 u64.
__global__ void __launch_bounds__(kTileThreads, 1) k1_zeta_low(LatticeDev *states)
{
	extern __shared__ unsigned long long sm[];
	__shared__ double ctab[kMaxClasses];
	__shared__ float red[32];
	__shared__ int s_flag;
	LatticeDev &L = states[blockIdx.y];
	const int tid = threadIdx.x;
	const int tbits = L.tbits;
	const int hbits = L.hbits;
	const unsigned int tsize = 1u << tbits;
	const unsigned int row = blockIdx.x;
	const unsigned long long base = static_cast<unsigned long long>(row) << tbits;
	const int mode = L.mode;
	const unsigned int e = L.pend_e;

	if (tid == 0)
		s_flag = 0;
	if (mode == kUpdate && tid < kMaxClasses)
	{
		const int pool = __popc(e);
		double c = 0.0;
		if (tid <= pool)
			c = binary_likelihood(L.dilution, pool, tid, L.pend_r, L.dil, L.orig_n + 1) / L.z_norm;
		ctab[tid] = c;
	}
	__syncthreads();

	// Phase A: x = tid + 1024 i (lattice bits 10..13 in registers).
	double v[kPerThread];
	float f = 0.0f;
	int bad = 0;
	const double *q_in = L.q_in;
	double *q_out = L.q_out;
#pragma unroll
	for (int i = 0; i < kPerThread; i++)
	{
		const unsigned int x = static_cast<unsigned int>(tid) + static_cast<unsigned int>(kTileThreads) * i;
		double val = 0.0;
		if (x < tsize)
		{
			const unsigned long long s = base | x;
			if (mode == kGenerate)
				val = L.prior_hi[row] * L.prior_lo[x];
			else
				val = q_in[s];
			if (mode == kUpdate)
				val *= ctab[__popc(e & static_cast<unsigned int>(s))];
			if (mode != kLoad)
				q_out[s] = val;
		}
		bad |= ((static_cast<unsigned long long>(__double_as_longlong(val)) >> 52) & 0x7FF) == 0x7FF;
		v[i] = val;
		f += approx_scaled(val);
	}
	if (bad)
		s_flag = 1;
	const float tile_est = block_sum_1024(f, red);
	// Scale so that the tile total lands in [2^61, 2^62 * (1 + 2^-22)).
	const int ef = (__float_as_int(tile_est) >> 23) & 0xFF;
	const int scale = ef == 0 ? 237 : 252 - ef;

	unsigned long long a[kPerThread];
#pragma unroll
	for (int i = 0; i < kPerThread; i++)
		a[i] = to_fixed(v[i], scale);
	reg_zeta16(a, 10, tbits);
#pragma unroll
	for (int i = 0; i < kPerThread; i++)
		sm[tile_swz(static_cast<unsigned int>(tid) + kTileThreads * i)] = a[i];
	__syncthreads();

	// Phase B: lattice bits 6..9 in registers.
	{
		const unsigned int xb = (tid & 63) | ((tid >> 6) << 10);
#pragma unroll
		for (int i = 0; i < kPerThread; i++)
			a[i] = sm[tile_swz(xb | (i << 6))];
		reg_zeta16(a, 6, tbits);
#pragma unroll
		for (int i = 0; i < kPerThread; i++)
			sm[tile_swz(xb | (i << 6))] = a[i];
	}
	__syncthreads();
	// Phase C: lattice bits 2..5 in registers.
	{
		const unsigned int xc = (tid & 3) | ((tid >> 2) << 6);
#pragma unroll
		for (int i = 0; i < kPerThread; i++)
			a[i] = sm[tile_swz(xc | (i << 2))];
		reg_zeta16(a, 2, tbits);
#pragma unroll
		for (int i = 0; i < kPerThread; i++)
			sm[tile_swz(xc | (i << 2))] = a[i];
	}
	__syncthreads();
	// Phase D: lattice bits 0..1 in registers; thread tid owns column block tid.
	{
		const unsigned int xd = static_cast<unsigned int>(tid) << 4;
#pragma unroll
		for (int i = 0; i < kPerThread; i++)
			a[i] = sm[tile_swz(xd | i)];
#pragma unroll
		for (int lvl = 0; lvl < 2; lvl++)
		{
			if (lvl < tbits)
			{
#pragma unroll
				for (int i = 0; i < kPerThread; i++)
					if (!(i & (1 << lvl)))
						a[i] += a[i | (1 << lvl)];
			}
		}
		if (xd < tsize || tid == 0)
		{
			const unsigned int rows = 1u << hbits;
			unsigned long long *dst = L.m1 + (static_cast<size_t>(tid) * rows + row) * kColW;
#pragma unroll
			for (int i = 0; i < kPerThread; i += 2)
				*reinterpret_cast<ulonglong2 *>(dst + i) = make_ulonglong2(a[i], a[i + 1]);
		}
		if (tid == 0)
		{
			L.tile_total[row] = a[0];
			L.tile_scale[row] = scale;
		}
	}

	// Last CTA of this lattice: global scale and exact total.
	__shared__ bool s_last;
	__syncthreads();
	if (tid == 0)
	{
		if (s_flag)
			atomicExch(&L.error, kErrNonFinite);
		__threadfence();
		const unsigned int prev = atomicAdd(&L.k1_count, 1u);
		s_last = prev == gridDim.x - 1;
	}
	__syncthreads();
	if (!s_last)
		return;
	__threadfence();
	const unsigned int rows = 1u << hbits;
	__shared__ double dred[32];
	__shared__ unsigned long long ured[32];
	double zr = 0.0;
	for (unsigned int rr = tid; rr < rows; rr += kTileThreads)
	{
		const unsigned long long t = __ldcg(L.tile_total + rr);
		const int sc = __ldcg(L.tile_scale + rr);
		zr += __ull2double_rn(t) * pow2_neg(sc);
	}
	for (int o = 16; o > 0; o >>= 1)
		zr += __shfl_xor_sync(0xFFFFFFFFu, zr, o);
	if ((tid & 31) == 0)
		dred[tid >> 5] = zr;
	__syncthreads();
	if (tid < 32)
	{
		double t = dred[tid];
		for (int o = 16; o > 0; o >>= 1)
			t += __shfl_xor_sync(0xFFFFFFFFu, t, o);
		if (tid == 0)
			dred[0] = t;
	}
	__syncthreads();
	const double z_real = dred[0];
	const int ez = static_cast<int>((static_cast<unsigned long long>(__double_as_longlong(z_real)) >> 52) & 0x7FF);
	const int s_g = 1084 - ez;
	unsigned long long zg = 0;
	for (unsigned int rr = tid; rr < rows; rr += kTileThreads)
		zg += rescale(__ldcg(L.tile_total + rr), s_g - __ldcg(L.tile_scale + rr));
	for (int o = 16; o > 0; o >>= 1)
		zg += __shfl_xor_sync(0xFFFFFFFFu, zg, o);
	__syncthreads();
	if ((tid & 31) == 0)
		ured[tid >> 5] = zg;
	__syncthreads();
	__shared__ unsigned long long s_zg;
	if (tid < 32)
	{
		unsigned long long t = ured[tid];
		for (int o = 16; o > 0; o >>= 1)
			t += __shfl_xor_sync(0xFFFFFFFFu, t, o);
		if (tid == 0)
			s_zg = t;
	}
	__syncthreads();
	// Exact atom marginals at the global scale: warp w sums atom w over the
	// tiles.  Low atoms read the singleton column 1 << w of every tile's
	// partial sums; high atoms add the totals of the tiles whose row index has
	// bit w - tbits set.
	{
		const int warp = tid >> 5, lane = tid & 31;
		if (warp < L.atoms)
		{
			unsigned long long acc = 0;
			if (warp < tbits)
			{
				const unsigned int col = 1u << warp;
				const unsigned long long *src = L.m1 + (static_cast<size_t>(col / kColW) * rows) * kColW + (col % kColW);
				for (unsigned int rr = lane; rr < rows; rr += 32)
					acc += rescale(__ldcg(src + static_cast<size_t>(rr) * kColW), s_g - __ldcg(L.tile_scale + rr));
			}
			else
			{
				const unsigned int hb = 1u << (warp - tbits);
				for (unsigned int rr = lane; rr < rows; rr += 32)
					if (rr & hb)
						acc += rescale(__ldcg(L.tile_total + rr), s_g - __ldcg(L.tile_scale + rr));
			}
			for (int o = 16; o > 0; o >>= 1)
				acc += __shfl_xor_sync(0xFFFFFFFFu, acc, o);
			if (lane == 0)
				L.atom_fixed[warp] = acc;
		}
	}
	__syncthreads();
	if (tid == 0)
	{
		__threadfence();
		const unsigned long long t = s_zg;
		L.s_g = s_g;
		L.z_g = t;
		if (t == 0 || ez == 0)
			atomicExch(&L.error, kErrZeroMass);
		if (mode == kUpdate)
			L.z_norm = __ull2double_rn(t) * pow2_neg(s_g);
		else if (mode == kGenerate)
			L.z_norm = 1.0;
		if (mode != kLoad)
			L.q_in = L.q_out;
		L.mode = kLoad;
		if (mode == kUpdate && L.classify_on_update)
		{
			classify_atoms(L, L.up, L.lo);
			if (L.sess_active)
			{
				const int st = L.stage;
				if (L.out_pos)
					L.out_pos[st - 1] = L.pos;
				if (L.out_neg)
					L.out_neg[st - 1] = L.neg;
				if (st >= L.stages)
					L.sess_active = 0;
			}
		}
		L.k1_count = 0;
	}
}

// ------------------------------------------------------------------ K2

__device__ __forceinline__ void argmin_warp(unsigned long long &s, unsigned int &e)
{
	for (int o = 16; o > 0; o >>= 1)
	{
		const unsigned long long os = __shfl_xor_sync(0xFFFFFFFFu, s, o);
		const unsigned int oe = __shfl_xor_sync(0xFFFFFFFFu, e, o);
		if (better(os, oe, s, e))
		{
			s = os;
			e = oe;
		}
	}
}

// One K2 column block: see the header.  Dynamic shared memory:
// 2^hbits * 16 u64 plus 2^hbits ints.
__global__ void __launch_bounds__(kHighThreads, 1) k2_zeta_high_select(LatticeDev *states)
{
	extern __shared__ unsigned long long sm[];
	LatticeDev &L = states[blockIdx.y];
	if (L.skip)
		return;
	const int tid = threadIdx.x;
	const int tbits = L.tbits, hbits = L.hbits;
	const unsigned int rows = 1u << hbits;
	const unsigned int b = blockIdx.x;
	int *shift = reinterpret_cast<int *>(sm + static_cast<size_t>(rows) * kColW);
	const int s_g = L.s_g;
	for (unsigned int rr = tid; rr < rows; rr += kHighThreads)
		shift[rr] = s_g - L.tile_scale[rr];
	__syncthreads();

	const unsigned int c = tid & 15;
	const unsigned int g = tid >> 4; // 0..31
	unsigned long long a[32];
	const unsigned long long *src = L.m1 + static_cast<size_t>(b) * rows * kColW;
	// Phase 1: rows g + 32 i (row bits 5..9 in registers).
#pragma unroll
	for (int i = 0; i < 32; i++)
	{
		const unsigned int rr = g + 32u * i;
		a[i] = rr < rows ? rescale(src[rr * kColW + c], shift[rr]) : 0ull;
	}
#pragma unroll
	for (int lvl = 0; lvl < 5; lvl++)
	{
		if (5 + lvl < hbits)
		{
#pragma unroll
			for (int i = 0; i < 32; i++)
				if (!(i & (1 << lvl)))
					a[i] += a[i | (1 << lvl)];
		}
	}
#pragma unroll
	for (int i = 0; i < 32; i++)
	{
		const unsigned int rr = g + 32u * i;
		if (rr < rows)
			sm[rr * kColW + c] = a[i];
	}
	__syncthreads();
	// Phase 2: rows 32 g + i (row bits 0..4 in registers), then score.
#pragma unroll
	for (int i = 0; i < 32; i++)
	{
		const unsigned int rr = 32u * g + i;
		a[i] = rr < rows ? sm[rr * kColW + c] : 0ull;
	}
#pragma unroll
	for (int lvl = 0; lvl < 5; lvl++)
	{
		if (lvl < hbits)
		{
#pragma unroll
			for (int i = 0; i < 32; i++)
				if (!(i & (1 << lvl)))
					a[i] += a[i | (1 << lvl)];
		}
	}
	const unsigned int e_lo = b * kColW + c;
	const unsigned long long zg = L.z_g;
	const unsigned int active = L.active;
	unsigned long long best = ~0ull;
	unsigned int best_e = 0xFFFFFFFFu;
	if (e_lo < (1u << tbits))
	{
#pragma unroll
		for (int i = 0; i < 32; i++)
		{
			const unsigned int rr = 32u * g + i;
			if (rr < rows)
			{
				const unsigned int E = (rr << tbits) | e_lo;
				const unsigned long long m2 = a[i] << 1;
				const unsigned long long score = m2 > zg ? m2 - zg : zg - m2;
				if ((E & ~active) == 0 && better(score, E, best, best_e))
				{
					best = score;
					best_e = E;
				}
			}
		}
	}
	argmin_warp(best, best_e);
	__shared__ unsigned long long wsc[kHighThreads / 32];
	__shared__ unsigned int wse[kHighThreads / 32];
	if ((tid & 31) == 0)
	{
		wsc[tid >> 5] = best;
		wse[tid >> 5] = best_e;
	}
	__syncthreads();
	__shared__ bool s_last;
	if (tid < 32)
	{
		unsigned long long s2 = tid < kHighThreads / 32 ? wsc[tid] : ~0ull;
		unsigned int e2 = tid < kHighThreads / 32 ? wse[tid] : 0xFFFFFFFFu;
		argmin_warp(s2, e2);
		if (tid == 0)
		{
			L.blk_score[b] = s2;
			L.blk_e[b] = e2;
			__threadfence();
			const unsigned int prev = atomicAdd(&L.k2_count, 1u);
			s_last = prev == gridDim.x - 1;
		}
	}
	__syncthreads();
	if (!s_last)
		return;
	__threadfence();
	unsigned long long bs = ~0ull;
	unsigned int be = 0xFFFFFFFFu;
	for (int i = tid; i < static_cast<int>(gridDim.x); i += kHighThreads)
	{
		const unsigned long long s2 = __ldcg(L.blk_score + i);
		const unsigned int e2 = __ldcg(L.blk_e + i);
		if (better(s2, e2, bs, be))
		{
			bs = s2;
			be = e2;
		}
	}
	argmin_warp(bs, be);
	__syncthreads();
	if ((tid & 31) == 0)
	{
		wsc[tid >> 5] = bs;
		wse[tid >> 5] = be;
	}
	__syncthreads();
	if (tid < 32)
	{
		unsigned long long s2 = tid < kHighThreads / 32 ? wsc[tid] : ~0ull;
		unsigned int e2 = tid < kHighThreads / 32 ? wse[tid] : 0xFFFFFFFFu;
		argmin_warp(s2, e2);
		if (tid == 0)
		{
			__threadfence();
			L.best_score = s2;
			L.best_e = e2;
			L.k2_count = 0;
			if (L.sess_active)
			{
				// Session step (bgt::Lattice order: select -> update -> classify).
				const int st = L.stage;
				if (st < L.stages)
				{
					const unsigned int r = bgt_session_sample_response(L.dilution, L.n, L.k, e2, L.truth, L.alpha,
																	   L.hpar, L.seed, L.session,
																	   static_cast<uint32_t>(st));
					if (L.out_e)
						L.out_e[st] = e2;
					if (L.out_r)
						L.out_r[st] = r;
					L.pend_e = e2;
					L.pend_r = r;
					L.mode = kUpdate;
					L.stage = st + 1;
				}
			}
		}
	}
}

// ------------------------------------------------------------------ misc

// Product-prior tables: lo[x] = prod over atoms 0..tbits-1, hi[r] = prod over
// atoms tbits..atoms-1, each in ascending atom order (prior_prob,
// src/core/model/lattice_base.cpp:197-208, split at bit tbits).
__global__ void prior_tables(const double *pi0, int atoms, int tbits, double *lo, double *hi)
{
	const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
	const unsigned int nlo = 1u << tbits, nhi = 1u << (atoms - tbits);
	if (i < nlo)
	{
		double p = 1.0;
		for (int a = 0; a < tbits; a++)
			p *= (i & (1u << a)) ? (1.0 - pi0[a]) : pi0[a];
		lo[i] = p;
	}
	if (i < nhi)
	{
		double p = 1.0;
		for (int a = tbits; a < atoms; a++)
			p *= (i & (1u << (a - tbits))) ? (1.0 - pi0[a]) : pi0[a];
		hi[i] = p;
	}
}

// Exact fixed-point upset mass sum_{s superset of e} q[s] at the lattice's
// global scale (for Lattice::upset_probability_mass).
__global__ void upset_mass_kernel(const LatticeDev *state, unsigned int e, unsigned long long *out)
{
	const LatticeDev &L = *state;
	const unsigned int free_bits = ~e & ((L.atoms >= 32) ? 0xFFFFFFFFu : ((1u << L.atoms) - 1u));
	const int nfree = __popc(free_bits);
	const unsigned long long count = 1ull << nfree;
	unsigned long long acc = 0;
	for (unsigned long long j = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; j < count;
		 j += static_cast<unsigned long long>(gridDim.x) * blockDim.x)
	{
		// Deposit the bits of j into the free positions.
		unsigned int s = e, fb = free_bits;
		unsigned long long jj = j;
		while (fb)
		{
			const unsigned int low = fb & (0u - fb);
			if (jj & 1ull)
				s |= low;
			jj >>= 1;
			fb ^= low;
		}
		acc += to_fixed(L.q_in[s], L.s_g);
	}
	for (int o = 16; o > 0; o >>= 1)
		acc += __shfl_xor_sync(0xFFFFFFFFu, acc, o);
	if ((threadIdx.x & 31) == 0)
		atomicAdd(out, acc);
}

} // namespace bgt_gpu
