/*
 * Counter-based random streams that define the synthetic adaptive-testing
 * workloads (seeded priors, true states, and the responses a session observes).
 *
 * Every value is a pure function of (seed, session, tag, index), so the GPU
 * session kernels, the host drivers and the CPU oracle draw identical
 * responses whenever they select identical experiments, whatever order or
 * batch the sessions run in.  The mixer is SplitMix64's finaliser (Steele,
 * Lea & Flood, "Fast splittable pseudorandom number generators", 2014).
 *
 * Bit conventions follow the reference lattice: atom = variant * subjects +
 * subject, state bit set = negative (healthy), response bit v set = the pool
 * tested negative for variant v.  No counterpart exists in the reference: it
 * takes responses from its caller.
 */
#ifndef BGT_SESSION_RNG_H
#define BGT_SESSION_RNG_H

#include <stdint.h>

#if defined(__CUDACC__)
#define BGT_RNG_FN static __host__ __device__ __forceinline__
#else
#define BGT_RNG_FN static inline
#endif

#define BGT_RNG_TAG_PRIOR 1u
#define BGT_RNG_TAG_TRUTH 2u
#define BGT_RNG_TAG_RESPONSE 3u
#define BGT_RNG_TAG_ARRIVAL 4u
#define BGT_RNG_TAG_SHAPE 5u

/* Probability that a non-dilution pool reports "negative" when every pooled
 * subject is negative, as hard-coded by the reference
 * (src/core/model/replicated_lattice.cpp:6). */
#define BGT_NON_DILUTION_NEGATIVE 0.99

BGT_RNG_FN uint64_t bgt_mix64(uint64_t z)
{
	z += 0x9E3779B97F4A7C15ull;
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
	return z ^ (z >> 31);
}

/* Uniform double in [0, 1) with 53 random bits. */
BGT_RNG_FN double bgt_uniform(uint64_t seed, uint64_t session, uint32_t tag, uint32_t index)
{
	const uint64_t key = bgt_mix64(seed ^ bgt_mix64(session + 0x632BE59BD9B4E019ull)) ^
						 bgt_mix64(((uint64_t)tag << 32) | (uint64_t)index);
	return (double)(bgt_mix64(key) >> 11) * (1.0 / 9007199254740992.0);
}

BGT_RNG_FN int bgt_popcount32(uint32_t v)
{
	v = v - ((v >> 1) & 0x55555555u);
	v = (v & 0x33333333u) + ((v >> 2) & 0x33333333u);
	return (int)((((v + (v >> 4)) & 0x0F0F0F0Fu) * 0x01010101u) >> 24);
}

/* Probability that response bit `variant` is 1 (pool negative) for
 * experiment e (subject mask) and true state s.  Non-dilution: `specificity`
 * when the pool is "contained" (all pooled subjects negative for the
 * variant), else 1 - `sensitivity`; the reference's model is
 * specificity = sensitivity = BGT_NON_DILUTION_NEGATIVE (0.99 and 0.01).
 * Dilution: the DilutionTable entry for pool size L and r positives in the
 * pool, alpha for r = 0 and 1 - alpha*r/((L-r)*h + r) otherwise; an empty
 * pool (L = 0) is given alpha, the r = 0 value. */
BGT_RNG_FN double bgt_response_bit_probability(int dilution, int subjects, uint32_t e, uint32_t s, int variant,
											   double alpha, double h, double specificity, double sensitivity)
{
	const uint32_t variant_state = (uint32_t)(((uint64_t)s) >> (variant * subjects));
	if (!dilution)
		return (e & variant_state) == e ? specificity : 1.0 - sensitivity;
	const int pool = bgt_popcount32(e);
	const int positives = pool - bgt_popcount32(e & variant_state);
	if (positives == 0)
		return alpha;
	const int negatives = pool - positives;
	return 1 - alpha * positives / (negatives * h + positives);
}

/* Response word for one stage of one session. */
BGT_RNG_FN uint32_t bgt_session_sample_response(int dilution, int subjects, int variants, uint32_t e, uint32_t s,
												double alpha, double h, double specificity, double sensitivity,
												uint64_t seed, uint64_t session, uint32_t stage)
{
	uint32_t response = 0;
	for (int v = 0; v < variants; v++)
	{
		const double p1 = bgt_response_bit_probability(dilution, subjects, e, s, v, alpha, h, specificity, sensitivity);
		const double u = bgt_uniform(seed, session, BGT_RNG_TAG_RESPONSE, stage * 64u + (uint32_t)v);
		if (u < p1)
			response |= 1u << v;
	}
	return response;
}

/* True state drawn from the product prior: atom i is positive (bit clear)
 * with probability pi0[i]. */
BGT_RNG_FN uint32_t bgt_session_sample_truth(int atoms, const double *pi0, uint64_t seed, uint64_t session)
{
	uint32_t state = 0;
	for (int i = 0; i < atoms; i++)
	{
		if (!(bgt_uniform(seed, session, BGT_RNG_TAG_TRUTH, (uint32_t)i) < pi0[i]))
			state |= 1u << i;
	}
	return state;
}

/* Per-atom prior prevalences drawn i.i.d. uniform in [lo, hi). */
BGT_RNG_FN void bgt_session_sample_prior(int atoms, double lo, double hi, uint64_t seed, uint64_t session, double *pi0)
{
	for (int i = 0; i < atoms; i++)
		pi0[i] = lo + (hi - lo) * bgt_uniform(seed, session, BGT_RNG_TAG_PRIOR, (uint32_t)i);
}

#endif
