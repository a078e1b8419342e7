// C entry points over the reference library's own CPU provider.
//
// Test infrastructure only: this file is compiled together with the
// reference's unmodified sources (see oracle/ref/Makefile) into
// oracle/_ref/libbgtref*.so, which the parity tests and the golden-vector
// script load with ctypes.  It lets those tests ask the *reference itself* for
// priors, updates, classifications, selections, tree statistics and whole
// adaptive sessions on seeded inputs.  All states, experiments and masks are
// in the reference's internal bit order (atom = variant * subjects + subject;
// bit set = negative).
//
// Lattice types follow the reference's internal enum
// (include/bgt/detail/internal_types.hpp:28-33): 3 = replicated non-dilution,
// 4 = replicated dilution.  Selectors follow bgt::SelectorType
// (include/bgt/types.hpp:89-94): 0 = auto, 1 = Op-BHA, 2 = Op-BBPA.

#include "bgt/bgt.hpp"
#include "bgt/detail/model/lattice.hpp"

#include <cstdint>
#include <cstring>
#include <exception>
#include <memory>
#include <span>
#include <vector>

#include "bgt_session_rng.h"

namespace
{

thread_local std::string g_last_error;

std::unique_ptr<bgt::model::Lattice> make_lattice(int type, int n, int k, const double *pi0, std::vector<double> &holder)
{
	holder.assign(pi0, pi0 + n * k);
	return bgt::model::create_lattice(static_cast<lattice_type_t>(type), n, k, holder.data());
}

void load_posterior(bgt::model::Lattice &lattice, const double *posterior)
{
	const int count = lattice.total_states();
	bgt::posterior_t *data = lattice.posterior_probs();
	for (int i = 0; i < count; i++)
		data[i] = static_cast<bgt::posterior_t>(posterior[i]);
}

void store_posterior(const bgt::model::Lattice &lattice, double *out)
{
	const int count = lattice.total_states();
	const bgt::posterior_t *data = lattice.posterior_probs();
	for (int i = 0; i < count; i++)
		out[i] = static_cast<double>(data[i]);
}

template <typename Fn>
int guarded(Fn &&fn)
{
	try
	{
		fn();
		return 0;
	}
	catch (const std::exception &error)
	{
		g_last_error = error.what();
		return 4;
	}
}

} // namespace

extern "C"
{

const char *ref_last_error() { return g_last_error.c_str(); }

int ref_posterior_bits() { return BGT_POSTERIOR_BITS; }

// Lattice::prior_probs (src/core/model/lattice_base.cpp:184-208).
int ref_prior(int type, int n, int k, const double *pi0, double *out)
{
	return guarded([&] {
		std::vector<double> holder;
		auto lattice = make_lattice(type, n, k, pi0, holder);
		store_posterior(*lattice, out);
	});
}

// DilutionTable (src/core/model/dilution.cpp:44-67): row-major n x (n+1).
int ref_dilution_table(int n, double alpha, double h, double *out)
{
	return guarded([&] {
		bgt::DilutionTable table(n, alpha, h);
		for (int row = 0; row < n; row++)
			for (int col = 0; col <= n; col++)
				out[row * (n + 1) + col] = col <= row + 1 ? table.rows()[row][col] : 0.0;
	});
}

// bgt::Lattice::select_experiments (src/core/lattice_api.cpp:116-168) through
// the public API: a binary non-dilution lattice from `pi0`, `nupd` updates in
// public order, then `count` experiments (public order).
int ref_select_experiments(int n, const double *pi0, int nupd, const uint32_t *upd_e, const uint32_t *upd_r,
						   int count, int selector, uint32_t *out)
{
	return guarded([&] {
		bgt::Lattice lattice(bgt::LatticeType::replicated_non_dilution, n, std::span<const double>(pi0, n));
		for (int i = 0; i < nupd; i++)
			lattice.update(upd_e[i], upd_r[i]);
		const std::vector<bgt::state_t> got = lattice.select_experiments(count, static_cast<bgt::SelectorType>(selector));
		for (std::size_t i = 0; i < got.size(); i++)
			out[i] = got[i];
	});
}

// response_prob (src/core/model/replicated_lattice.cpp:8-28).
int ref_response_prob(int type, int n, int k, const double *pi0, uint32_t e, uint32_t r, uint32_t s,
					  double alpha, double h, double *out)
{
	return guarded([&] {
		std::vector<double> holder;
		auto lattice = make_lattice(type, n, k, pi0, holder);
		bgt::DilutionTable table(n, alpha, h);
		*out = lattice->response_prob(e, r, s, type == 4 ? table.rows() : nullptr);
	});
}

// update_probs (lattice_base.cpp:210-228) when in_place == 0,
// update_probs_in_place (lattice_base.cpp:230-244) otherwise.
int ref_update(int type, int n, int k, const double *pi0, const double *post_in, uint32_t e, uint32_t r,
			   double alpha, double h, int in_place, double *post_out)
{
	return guarded([&] {
		std::vector<double> holder;
		auto lattice = make_lattice(type, n, k, pi0, holder);
		load_posterior(*lattice, post_in);
		bgt::DilutionTable table(n, alpha, h);
		double **rows = type == 4 ? table.rows() : nullptr;
		if (in_place)
			lattice->update_probs_in_place(e, r, rows);
		else
			lattice->update_probs(e, r, rows);
		store_posterior(*lattice, post_out);
	});
}

// get_atom_prob_mass (lattice_base.cpp:354-366) for every atom.
int ref_atom_masses(int type, int n, int k, const double *pi0, const double *post, double *masses)
{
	return guarded([&] {
		std::vector<double> holder;
		auto lattice = make_lattice(type, n, k, pi0, holder);
		load_posterior(*lattice, post);
		for (int atom = 0; atom < n * k; atom++)
			masses[atom] = lattice->get_atom_prob_mass(bgt::state_bit(atom));
	});
}

// get_prob_mass (lattice_base.cpp:319-351): upset mass of one experiment.
int ref_upset_mass(int type, int n, int k, const double *pi0, const double *post, uint32_t e, double *out)
{
	return guarded([&] {
		std::vector<double> holder;
		auto lattice = make_lattice(type, n, k, pi0, holder);
		load_posterior(*lattice, post);
		*out = lattice->get_prob_mass(e);
	});
}

// Lattice::select_experiment (src/kernels/cpu/bbpa.cpp:861-871).
int ref_select(int type, int n, int k, const double *pi0, const double *post, int selector, uint32_t *out)
{
	return guarded([&] {
		std::vector<double> holder;
		auto lattice = make_lattice(type, n, k, pi0, holder);
		load_posterior(*lattice, post);
		*out = lattice->select_experiment(static_cast<bgt::SelectorType>(selector));
	});
}

// update_metadata (lattice_base.cpp:246-264): classification masks in/out.
int ref_classify(int type, int n, int k, const double *pi0, const double *post, double up, double lo,
				 uint32_t *pos_mask, uint32_t *neg_mask)
{
	return guarded([&] {
		std::vector<double> holder;
		auto lattice = make_lattice(type, n, k, pi0, holder);
		load_posterior(*lattice, post);
		// The masks are protected members, so classify on a fresh lattice and
		// merge: update_metadata never revisits a classified atom and each
		// atom's decision depends only on its own mass, so keeping the incoming
		// masks and adding only the newly decided atoms is the same result.
		const uint32_t pos = *pos_mask, neg = *neg_mask;
		lattice->update_metadata(up, lo);
		uint32_t new_pos = lattice->pos_clas_atoms();
		uint32_t new_neg = lattice->neg_clas_atoms();
		const uint32_t already = pos | neg;
		*pos_mask = pos | (new_pos & ~already);
		*neg_mask = neg | (new_neg & ~already);
	});
}

// bgt::run_simulation with Provider::cpu (src/runtime/simulation_runner.cpp:181-262).
// out[0] = total_leaves, out[1..7] = the TreeStats probabilities in declaration order.
int ref_run_simulation(int type, int n, int k, const double *pi0, int depth, double up, double lo,
					   double branch, int selector, double alpha, double h, double *out)
{
	return guarded([&] {
		bgt::SimulationConfig config;
		config.lattice_type = type == 4 ? bgt::LatticeType::replicated_dilution : bgt::LatticeType::replicated_non_dilution;
		config.subjects = n;
		config.variants = k;
		config.prior.assign(pi0, pi0 + n * k);
		config.options.search_depth = depth;
		config.options.threshold_up = up;
		config.options.threshold_lo = lo;
		config.options.branch_threshold = branch;
		config.options.selector = static_cast<bgt::SelectorType>(selector);
		config.options.provider = bgt::Provider::cpu;
		config.dilution.alpha = alpha;
		config.dilution.h = h;
		const bgt::TreeStats stats = bgt::run_simulation(config).stats;
		out[0] = stats.total_leaves;
		out[1] = stats.correct_probability;
		out[2] = stats.incorrect_probability;
		out[3] = stats.false_positive_probability;
		out[4] = stats.false_negative_probability;
		out[5] = stats.unclassified_probability;
		out[6] = stats.expected_stages;
		out[7] = stats.expected_tests;
	});
}

// One adaptive session through the reference's model lattice: per stage
// select_experiment -> sampled response -> update_probs_in_place ->
// update_metadata, i.e. the bgt::Lattice session calls of
// src/core/lattice_api.cpp:108-178 in internal bit order.  The response to
// each stage is drawn from the session's own counter-based stream
// (session_rng.h) given the session's true state.  Runs `stages` stages
// unconditionally (the session API has no stopping rule).  Writes the
// selected experiments, responses and masks per stage and the final posterior.
int ref_session(int type, int n, int k, const double *pi0, int selector, double alpha, double h,
				double up, double lo, int stages, uint64_t seed, uint64_t session, uint32_t true_state,
				uint32_t *experiments, uint32_t *responses, uint32_t *pos_masks, uint32_t *neg_masks,
				double *final_post)
{
	return guarded([&] {
		std::vector<double> holder;
		auto lattice = make_lattice(type, n, k, pi0, holder);
		bgt::DilutionTable table(n, alpha, h);
		double **rows = type == 4 ? table.rows() : nullptr;
		for (int stage = 0; stage < stages; stage++)
		{
			const uint32_t e = lattice->select_experiment(static_cast<bgt::SelectorType>(selector));
			const uint32_t r = bgt_session_sample_response(type == 4, n, k, e, true_state, alpha, h, BGT_NON_DILUTION_NEGATIVE,
														   BGT_NON_DILUTION_NEGATIVE, seed, session,
														   static_cast<uint32_t>(stage));
			lattice->update_probs_in_place(e, r, rows);
			lattice->update_metadata(up, lo);
			experiments[stage] = e;
			responses[stage] = r;
			pos_masks[stage] = lattice->pos_clas_atoms();
			neg_masks[stage] = lattice->neg_clas_atoms();
		}
		store_posterior(*lattice, final_post);
	});
}

} // extern "C"
