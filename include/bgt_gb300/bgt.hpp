// C++20 host API of the GB300 provider, with the reference's public names:
// bgt::Lattice (include/bgt/lattice.hpp:34-67), bgt::DilutionTable
// (:17-32), bgt::TreeStats / SimulationOptions (include/bgt/types.hpp:81-130),
// bgt::run_simulation for local trees (include/bgt/simulation.hpp:127) and
// bgt::Error with bgt::StatusCode (include/bgt/status.hpp:10-60).  Code
// written against the reference's bgt::Lattice compiles against this header
// and runs on the device, through the C ABI of bgt_gpu.h and bgt_serve.h
// (link libbgt_gb300.so).
//
// Header-only: every method forwards to one C-ABI call and turns a non-zero
// status into bgt::Error (1 -> invalid_argument, 2 -> unsupported,
// 4 -> cuda_error), the way the reference's CUDA provider reports failures
// (include/bgt/detail/cuda_checks.hpp:12-24).  Binary lattices keep the
// reference's public subject order, the bit reversal of
// src/core/lattice_api.cpp:17-26.
#pragma once

#include <cstdint>
#include <span>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../bgt_gpu.h"
#include "../bgt_serve.h"

namespace bgt
{

using state_t = std::uint32_t;
using host_probability_t = double;

enum class LatticeType
{
	distributed_non_dilution,
	distributed_dilution,
	replicated_non_dilution,
	replicated_dilution
};

enum class SelectorType
{
	auto_select,
	op_bha,
	op_bbpa
};

enum class Provider
{
	auto_select,
	cpu,
	cuda
};

enum class Precision
{
	float32,
	float64
};

enum class StatusCode
{
	success,
	invalid_argument,
	unsupported,
	runtime_error,
	mpi_error,
	cuda_error,
	internal_error
};

class Error : public std::runtime_error
{
  public:
	Error(StatusCode code, const std::string &message) : std::runtime_error(message), code_(code) {}
	StatusCode code() const { return code_; }

  private:
	StatusCode code_;
};

namespace detail
{

inline void check(int status)
{
	if (status == BGT_GPU_OK)
		return;
	const char *msg = bgt_gpu_last_error();
	const std::string text = msg ? msg : "GB300 provider failure";
	if (status == BGT_GPU_MISSING_DILUTION)
		throw Error(StatusCode::invalid_argument, text);
	if (status == BGT_GPU_UNSUPPORTED)
		throw Error(StatusCode::unsupported, text);
	throw Error(StatusCode::cuda_error, text);
}

inline state_t reverse_bits(state_t value, int width)
{
	state_t out = 0;
	for (int i = 0; i < width; i++)
		out = (out << 1) | ((value >> i) & 1u);
	return out;
}

inline bool uses_dilution(LatticeType type)
{
	return type == LatticeType::replicated_dilution || type == LatticeType::distributed_dilution;
}

} // namespace detail

// DilutionTable(subjects, alpha, h): row L - 1 holds P(negative | L pooled,
// r positive) for r = 0..L (src/core/model/dilution.cpp:44-67).
class DilutionTable
{
  public:
	DilutionTable() = default;
	DilutionTable(int subjects, host_probability_t alpha, host_probability_t h) : subjects_(subjects)
	{
		if (subjects <= 0)
			throw std::invalid_argument("subjects must be positive.");
		values_.assign(static_cast<std::size_t>(subjects) * static_cast<std::size_t>(subjects + 1), 0.0);
		rows_.resize(static_cast<std::size_t>(subjects));
		for (int rk = 1; rk <= subjects; rk++)
		{
			double *row = values_.data() + static_cast<std::size_t>(rk - 1) * static_cast<std::size_t>(subjects + 1);
			rows_[static_cast<std::size_t>(rk - 1)] = row;
			row[0] = alpha;
			for (int r = 1; r <= rk; r++)
			{
				const int k = rk - r;
				row[r] = 1 - alpha * r / (k * h + r);
			}
		}
	}
	DilutionTable(const DilutionTable &o) : subjects_(o.subjects_), values_(o.values_) { rebind(); }
	DilutionTable &operator=(const DilutionTable &o)
	{
		subjects_ = o.subjects_;
		values_ = o.values_;
		rebind();
		return *this;
	}

	int subjects() const { return subjects_; }
	host_probability_t **rows() { return rows_.empty() ? nullptr : rows_.data(); }
	host_probability_t *const *rows() const { return rows_.empty() ? nullptr : rows_.data(); }
	host_probability_t at(int group_size, int positives) const
	{
		if (group_size <= 0 || group_size > subjects_ || positives < 0 || positives > group_size)
			throw std::out_of_range("dilution table index is out of range.");
		return rows_[static_cast<std::size_t>(group_size - 1)][positives];
	}

  private:
	void rebind()
	{
		rows_.resize(static_cast<std::size_t>(subjects_));
		for (int i = 0; i < subjects_; i++)
			rows_[static_cast<std::size_t>(i)] = values_.data() + static_cast<std::size_t>(i) * (subjects_ + 1);
	}
	int subjects_ = 0;
	std::vector<host_probability_t> values_;
	std::vector<host_probability_t *> rows_;
};

// bgt::Lattice on the device (src/core/lattice_api.cpp:61-196 is the CPU
// counterpart).
class Lattice
{
  public:
	Lattice(LatticeType type, int subjects, std::span<const host_probability_t> prior,
			Precision precision = Precision::float64)
		: Lattice(type, subjects, 1, prior, precision)
	{
	}
	Lattice(LatticeType type, int subjects, int variants, std::span<const host_probability_t> prior,
			Precision precision = Precision::float64)
		: type_(type), subjects_(subjects), variants_(variants)
	{
		if (subjects <= 0 || variants <= 0)
			throw Error(StatusCode::invalid_argument, "subjects and variants must be positive.");
		if (prior.size() != static_cast<std::size_t>(subjects) * static_cast<std::size_t>(variants))
			throw Error(StatusCode::invalid_argument, "prior length must equal subjects * variants.");
		if (type == LatticeType::distributed_non_dilution || type == LatticeType::distributed_dilution)
			throw Error(StatusCode::unsupported, "distributed lattices are not served by the GB300 provider.");
		detail::check(bgt_gpu_lattice_create(detail::uses_dilution(type) ? 1 : 0, subjects, variants, prior.data(),
											 precision == Precision::float32 ? BGT_GPU_FP32 : BGT_GPU_FP64, &h_));
	}
	~Lattice()
	{
		if (h_)
			bgt_gpu_lattice_destroy(h_);
	}
	Lattice(const Lattice &) = delete;
	Lattice &operator=(const Lattice &) = delete;
	Lattice(Lattice &&o) noexcept { *this = std::move(o); }
	Lattice &operator=(Lattice &&o) noexcept
	{
		if (this != &o)
		{
			if (h_)
				bgt_gpu_lattice_destroy(h_);
			h_ = std::exchange(o.h_, nullptr);
			type_ = o.type_;
			subjects_ = o.subjects_;
			variants_ = o.variants_;
			pos_ = o.pos_;
			neg_ = o.neg_;
		}
		return *this;
	}

	int subjects() const { return subjects_; }
	int variants() const { return variants_; }
	LatticeType type() const { return type_; }

	host_probability_t posterior_probability(state_t state) const
	{
		double out = 0.0;
		detail::check(bgt_gpu_lattice_posterior_probability(h_, to_internal(state), &out));
		return out;
	}
	host_probability_t upset_probability_mass(state_t experiment) const
	{
		double out = 0.0;
		detail::check(bgt_gpu_lattice_upset_mass(h_, to_internal(experiment), &out));
		return out;
	}
	state_t select_experiment(SelectorType selector = SelectorType::auto_select) const
	{
		uint32_t e = 0;
		detail::check(bgt_gpu_lattice_select(h_, static_cast<int>(selector), &e));
		return to_internal(e);
	}
	void update(state_t experiment, state_t response, const DilutionTable *dilution = nullptr)
	{
		if (detail::uses_dilution(type_) && dilution == nullptr)
			throw Error(StatusCode::invalid_argument, "dilution table is required for dilution models.");
		detail::check(bgt_gpu_lattice_update(h_, to_internal(experiment), response,
											 dilution ? dilution->rows() : nullptr));
	}
	void update_classification(host_probability_t threshold_up, host_probability_t threshold_lo)
	{
		detail::check(bgt_gpu_lattice_classify(h_, threshold_up, threshold_lo, &pos_, &neg_));
	}
	state_t positive_classification_mask() const { return to_internal(pos_); }
	state_t negative_classification_mask() const { return to_internal(neg_); }
	bool is_classified() const
	{
		return __builtin_popcount(pos_ | neg_) == subjects_ * variants_;
	}

	// The device handle, for the C ABI's session and comparison calls.
	bgt_gpu_lattice *native() { return h_; }

  private:
	// Internal <-> public order: reversed for binary lattices (an involution).
	state_t to_internal(state_t v) const { return variants_ == 1 ? detail::reverse_bits(v, subjects_) : v; }

	bgt_gpu_lattice *h_ = nullptr;
	LatticeType type_ = LatticeType::replicated_non_dilution;
	int subjects_ = 0, variants_ = 1;
	uint32_t pos_ = 0, neg_ = 0;
};

struct TreeStats
{
	int total_leaves = 0;
	double correct_probability = 0.0;
	double incorrect_probability = 0.0;
	double false_positive_probability = 0.0;
	double false_negative_probability = 0.0;
	double unclassified_probability = 0.0;
	double expected_stages = 0.0;
	double expected_tests = 0.0;
};

struct SimulationOptions
{
	int search_depth = 1;
	host_probability_t threshold_up = 0.01;
	host_probability_t threshold_lo = 0.01;
	double branch_threshold = 0.0;
	SelectorType selector = SelectorType::auto_select;
	Provider provider = Provider::auto_select;
};

struct DilutionParameters
{
	host_probability_t alpha = 0.99;
	host_probability_t h = 0.005;
};

// The local_tree subset of bgt::SimulationConfig (include/bgt/simulation.hpp:87-103).
struct SimulationConfig
{
	LatticeType lattice_type = LatticeType::replicated_non_dilution;
	int subjects = 0;
	int variants = 1;
	std::vector<host_probability_t> prior;
	SimulationOptions options;
	DilutionParameters dilution;
};

struct SimulationResult
{
	TreeStats stats;
	Provider provider = Provider::cuda;
	std::uint64_t total_states = 0;
	std::uint64_t evaluated_states = 0;
};

inline bool cuda_available() { return bgt_cuda_provider_available() != 0; }

// bgt::run_simulation for local trees on the device (Runtime::run_simulation,
// src/runtime/simulation_runner.cpp:181-262, through CudaProvider::run).
inline SimulationResult run_simulation(const SimulationConfig &config)
{
	const SimulationOptions &o = config.options;
	if (config.subjects <= 0 || config.variants <= 0 || o.search_depth < 0)
		throw Error(StatusCode::invalid_argument, "invalid simulation dimensions.");
	if (config.prior.size() != static_cast<std::size_t>(config.subjects) * static_cast<std::size_t>(config.variants))
		throw Error(StatusCode::invalid_argument, "prior length must equal subjects * variants.");
	if (o.provider == Provider::cpu)
		throw Error(StatusCode::unsupported, "the CPU provider is the reference library's.");
	const bool dil = detail::uses_dilution(config.lattice_type);
	DilutionTable table;
	if (dil)
		table = DilutionTable(config.subjects, config.dilution.alpha, config.dilution.h);
	bgt_tree_stats st{};
	detail::check(bgt_cuda_provider_run(dil ? 1 : 0, config.subjects, config.variants, config.prior.data(),
										o.search_depth, o.threshold_up, o.threshold_lo, o.branch_threshold,
										static_cast<int>(o.selector), dil ? table.rows() : nullptr, &st));
	SimulationResult r;
	r.stats = TreeStats{st.total_leaves,
						st.correct_probability,
						st.incorrect_probability,
						st.false_positive_probability,
						st.false_negative_probability,
						st.unclassified_probability,
						st.expected_stages,
						st.expected_tests};
	r.total_states = r.evaluated_states = std::uint64_t{1} << (config.subjects * config.variants);
	return r;
}

} // namespace bgt
