// C++20 host API of the GB300 provider, with the reference's public names:
// bgt::Lattice (include/bgt/lattice.hpp:34-67), bgt::DilutionTable
// (:17-32), bgt::TreeStats / SimulationOptions (include/bgt/types.hpp:81-130),
// bgt::run_simulation for local trees with its run report, progress snapshots
// and cancellation (include/bgt/simulation.hpp:13-129) and bgt::Error with
// bgt::StatusCode (include/bgt/status.hpp:10-60).  Code
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

#include <atomic>
#include <cctype>
#include <cstdlib>
#include <chrono>
#include <cstdint>
#include <filesystem>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <mutex>
#include <optional>
#include <span>
#include <sstream>
#include <stdexcept>
#include <string>
#include <string_view>
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

// include/bgt/compile_options.hpp:11-93 and include/bgt/types.hpp:103-107.
// The device kernels are compiled once for sm_103a; CompileOptions and
// KernelSpec are kept so that code building them compiles unchanged, and a
// KernelSpec records what a run asked for.
enum class OptimizationLevel
{
	debug,
	release,
	aggressive
};

enum class ProfileBackend
{
	none,
	caliper
};

enum class DilutionMode
{
	non_dilution,
	dilution
};

struct CompileOptions
{
	bool enable_simd = false;
	bool enable_openmp = false;
	bool enable_cuda = true;
	bool enable_nccl = false;
	bool enable_nccl_gin = false;
	bool fast_math = false;
	bool native_cpu = false;
	Precision posterior_precision = Precision::float64;
	Precision accumulator_precision = Precision::float64;
	OptimizationLevel optimization = OptimizationLevel::release;
	ProfileBackend profile_backend = ProfileBackend::none;
	std::vector<std::string> extra_cxx_flags;
	std::vector<std::string> extra_cuda_flags;
	std::vector<std::string> definitions;

	bool operator==(const CompileOptions &) const = default;
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
	// Lattice::select_experiments (src/core/lattice_api.cpp:116-168): the
	// Op-BHA selection, then greedy lookahead candidates (public order).
	std::vector<state_t> select_experiments(int k, SelectorType selector = SelectorType::op_bha) const
	{
		if (k < 0)
			throw std::invalid_argument("k must be non-negative.");
		std::vector<state_t> out(static_cast<std::size_t>(k));
		if (k == 0)
			return out;
		std::vector<uint32_t> raw(static_cast<std::size_t>(k));
		const int rc = bgt_gpu_lattice_select_experiments(h_, k, static_cast<int>(selector), raw.data());
		if (rc == BGT_GPU_MISSING_DILUTION)
			throw std::invalid_argument(bgt_gpu_last_error());
		detail::check(rc);
		for (std::size_t i = 0; i < out.size(); i++)
			out[i] = to_internal(raw[i]);
		return out;
	}
	// Extension: the non-dilution likelihood of later updates
	// (bgt_gpu_lattice_set_test_accuracy).
	void set_test_accuracy(host_probability_t sensitivity, host_probability_t specificity)
	{
		detail::check(bgt_gpu_lattice_set_test_accuracy(h_, sensitivity, specificity));
	}
	host_probability_t response_probability(state_t experiment, state_t response, state_t true_state,
										  const DilutionTable *dilution = nullptr) const
	{
		double out = 0.0;
		detail::check(bgt_gpu_lattice_response_probability(
			h_, to_internal(experiment), response, to_internal(true_state),
			dilution ? const_cast<host_probability_t **>(dilution->rows()) : nullptr, &out));
		return out;
	}
	state_t select_experiment(SelectorType selector = SelectorType::auto_select) const
	{
		// Model-level check of Lattice::select_experiment (src/kernels/cpu/bbpa.cpp:864-867).
		if (selector == SelectorType::op_bha && variants_ != 1)
			throw std::invalid_argument("Op-BHA experiment selection is only supported for binary lattices.");
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
	CompileOptions compile_options;
};

struct DilutionParameters
{
	host_probability_t alpha = 0.99;
	host_probability_t h = 0.005;
};

// include/bgt/simulation.hpp:13-42.  Only local_tree is served here; the
// parallel modes need the MPI backend.
enum class SimulationMode
{
	local_tree,
	parallel_global_tree,
	parallel_dynamic_tree,
	parallel_hybrid_tree,
	parallel_partial_tree,
	parallel_fusion_tree
};

enum class TrueStatePolicy
{
	all,
	trimmed,
	symmetric
};

enum class SimulationRunStatus
{
	completed,
	interrupted,
	running
};

enum class TerminationReason
{
	none,
	user_signal,
	cancellation_requested
};

// include/bgt/simulation.hpp:50-72.
struct ReportConfig
{
	bool write_csv = false;
	std::filesystem::path output_directory = ".";
	std::string run_name;
};

struct SimulationTimings
{
	double setup_seconds = 0.0;
	double tree_build_seconds = 0.0;
	double evaluation_seconds = 0.0;
	double total_seconds = 0.0;
};

struct ProgressConfig
{
	bool enabled = false;
	double interval_seconds = 5.0;
	std::filesystem::path output_path;
	bool write_jsonl = true;
	bool print_stderr = false;
};

// bgt::SimulationConfig (include/bgt/simulation.hpp:87-103).  As on the
// reference's CUDA path, evaluation_prior, true_state_policy, trim_percent,
// global_tree_depth and workload_granularity do not change a local_tree run on
// the device (every true state is evaluated under the prior).
// bgt::ProgressSnapshot (include/bgt/simulation.hpp:74-85): one progress record.
struct ProgressSnapshot
{
	SimulationRunStatus status = SimulationRunStatus::completed;
	TerminationReason reason = TerminationReason::none;
	int total_states = 0;
	int evaluated_states = 0;
	double state_coverage_fraction = 0.0;
	host_probability_t evaluated_prior_mass = 0.0;
	TreeStats stats;
	SimulationTimings timings;
	std::string message;
};

// Non-dilution test accuracy, an extension: the reference fixes both at 0.99
// (src/core/model/replicated_lattice.cpp:6-14).  P(negative response | no
// pooled positive) = specificity, P(positive response | a pooled positive) =
// sensitivity, per variant.
struct TestAccuracy
{
	host_probability_t sensitivity = 0.99;
	host_probability_t specificity = 0.99;
};

struct SimulationConfig
{
	LatticeType lattice_type = LatticeType::replicated_non_dilution;
	int subjects = 0;
	int variants = 1;
	std::vector<host_probability_t> prior;
	std::optional<std::vector<host_probability_t>> evaluation_prior;
	SimulationOptions options;
	SimulationMode mode = SimulationMode::local_tree;
	TrueStatePolicy true_state_policy = TrueStatePolicy::all;
	int global_tree_depth = 0;
	int workload_granularity = 1;
	host_probability_t trim_percent = 1.0;
	DilutionParameters dilution;
	ReportConfig report;
	ProgressConfig progress;
	std::optional<TestAccuracy> test_accuracy; // extension; unset = the reference's model
};

// bgt::KernelSpec (include/bgt/types.hpp:132-181): what a run asks for.
struct KernelSpec
{
	Provider provider = Provider::auto_select;
	int subjects = 0;
	int variants = 1;
	int state_bits = 32;
	DilutionMode dilution = DilutionMode::non_dilution;
	SelectorType selector = SelectorType::auto_select;
	Precision precision = Precision::float64;
	Precision accumulator_precision = Precision::float64;
	std::string cuda_arch = "sm_103a";
	CompileOptions compile_options;

	bool operator==(const KernelSpec &) const = default;
};

struct KernelSpecHash
{
	std::size_t operator()(const KernelSpec &spec) const
	{
		std::size_t seed = 0;
		auto mix = [&seed](std::size_t v) { seed ^= v + 0x9e3779b9u + (seed << 6) + (seed >> 2); };
		mix(static_cast<std::size_t>(spec.provider));
		mix(static_cast<std::size_t>(spec.subjects));
		mix(static_cast<std::size_t>(spec.variants));
		mix(static_cast<std::size_t>(spec.state_bits));
		mix(static_cast<std::size_t>(spec.dilution));
		mix(static_cast<std::size_t>(spec.selector));
		mix(static_cast<std::size_t>(spec.precision));
		mix(static_cast<std::size_t>(spec.accumulator_precision));
		mix(std::hash<std::string>{}(spec.cuda_arch));
		return seed;
	}
};

// bgt::JitCacheInfo (include/bgt/types.hpp:183-189): no run-time compilation
// here, so always empty and disabled.
struct JitCacheInfo
{
	std::size_t memory_entries = 0;
	std::size_t disk_entries = 0;
	std::string disk_cache_directory;
	bool jit_enabled = false;
};

// bgt::SimulationResult (include/bgt/simulation.hpp:105-121).
struct SimulationResult
{
	TreeStats stats;
	KernelSpec kernel;
	SimulationMode mode = SimulationMode::local_tree;
	Provider provider = Provider::auto_select;
	int rank = 0;
	int world_size = 1;
	int total_states = 0;
	int evaluated_states = 0;
	std::string report_path;
	SimulationTimings timings;
	SimulationRunStatus status = SimulationRunStatus::completed;
	TerminationReason termination_reason = TerminationReason::none;
	host_probability_t evaluated_prior_mass = 0.0;
	std::string progress_path;
};

// Cancellation (src/runtime/progress.cpp:82-108): the first request wins.
namespace detail
{
inline std::atomic<int> cancel_reason{static_cast<int>(TerminationReason::none)};
} // namespace detail

inline void clear_simulation_cancellation()
{
	detail::cancel_reason.store(static_cast<int>(TerminationReason::none), std::memory_order_release);
}

inline void request_simulation_cancellation(TerminationReason reason = TerminationReason::cancellation_requested)
{
	if (reason == TerminationReason::none)
		reason = TerminationReason::cancellation_requested;
	int expected = static_cast<int>(TerminationReason::none);
	detail::cancel_reason.compare_exchange_strong(expected, static_cast<int>(reason), std::memory_order_acq_rel);
}

inline bool simulation_cancellation_requested()
{
	return detail::cancel_reason.load(std::memory_order_acquire) != static_cast<int>(TerminationReason::none);
}

inline TerminationReason simulation_cancellation_reason()
{
	return static_cast<TerminationReason>(detail::cancel_reason.load(std::memory_order_acquire));
}

namespace detail
{

inline const char *mode_name(SimulationMode mode)
{
	switch (mode)
	{
	case SimulationMode::local_tree:
		return "local_tree";
	case SimulationMode::parallel_global_tree:
		return "parallel_global_tree";
	case SimulationMode::parallel_dynamic_tree:
		return "parallel_dynamic_tree";
	case SimulationMode::parallel_hybrid_tree:
		return "parallel_hybrid_tree";
	case SimulationMode::parallel_partial_tree:
		return "parallel_partial_tree";
	case SimulationMode::parallel_fusion_tree:
		return "parallel_fusion_tree";
	}
	return "unknown";
}

inline const char *status_name(SimulationRunStatus status)
{
	switch (status)
	{
	case SimulationRunStatus::completed:
		return "completed";
	case SimulationRunStatus::interrupted:
		return "interrupted";
	case SimulationRunStatus::running:
		return "running";
	}
	return "unknown";
}

inline const char *reason_name(TerminationReason reason)
{
	switch (reason)
	{
	case TerminationReason::none:
		return "none";
	case TerminationReason::user_signal:
		return "user_signal";
	case TerminationReason::cancellation_requested:
		return "cancellation_requested";
	}
	return "unknown";
}

inline std::string run_name(const SimulationConfig &config)
{
	return config.report.run_name.empty() ? mode_name(config.mode) : config.report.run_name;
}

inline double seconds_since(std::chrono::steady_clock::time_point start)
{
	return std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
}

} // namespace detail

// The field,value report of a finished (or interrupted: .partial.csv) run,
// or "" when none was asked for; the fields and their iostream formatting
// follow write_report_if_requested (src/runtime/reporting.cpp:10-45).
inline std::string write_report_if_requested(const SimulationConfig &config, const SimulationResult &result)
{
	if (!config.report.write_csv || result.rank != 0)
		return {};
	std::filesystem::create_directories(config.report.output_directory);
	const bool partial = result.status == SimulationRunStatus::interrupted;
	const std::filesystem::path path =
		config.report.output_directory / (detail::run_name(config) + (partial ? ".partial.csv" : ".csv"));
	std::ofstream out(path, std::ios::trunc);
	const TreeStats &st = result.stats;
	const SimulationTimings &tm = result.timings;
	const double coverage = result.total_states == 0 ? 0.0
													 : static_cast<double>(result.evaluated_states) /
														   static_cast<double>(result.total_states);
	out << "field,value\n"
		<< "status," << detail::status_name(result.status) << '\n'
		<< "termination_reason," << detail::reason_name(result.termination_reason) << '\n'
		<< "is_partial," << (partial ? "true" : "false") << '\n'
		<< "mode," << detail::mode_name(result.mode) << '\n'
		<< "provider," << static_cast<int>(result.provider) << '\n'
		<< "subjects," << config.subjects << '\n'
		<< "variants," << config.variants << '\n'
		<< "world_size," << result.world_size << '\n'
		<< "total_states," << result.total_states << '\n'
		<< "evaluated_states," << result.evaluated_states << '\n'
		<< "state_coverage_fraction," << coverage << '\n'
		<< "evaluated_prior_mass," << result.evaluated_prior_mass << '\n'
		<< "progress_path," << result.progress_path << '\n'
		<< "total_leaves," << st.total_leaves << '\n'
		<< "correct_probability," << st.correct_probability << '\n'
		<< "incorrect_probability," << st.incorrect_probability << '\n'
		<< "false_positive_probability," << st.false_positive_probability << '\n'
		<< "false_negative_probability," << st.false_negative_probability << '\n'
		<< "unclassified_probability," << st.unclassified_probability << '\n'
		<< "expected_stages," << st.expected_stages << '\n'
		<< "expected_tests," << st.expected_tests << '\n'
		<< "setup_seconds," << tm.setup_seconds << '\n'
		<< "tree_build_seconds," << tm.tree_build_seconds << '\n'
		<< "evaluation_seconds," << tm.evaluation_seconds << '\n'
		<< "total_seconds," << tm.total_seconds << '\n';
	return path.string();
}

namespace detail
{

inline std::string json_escape(const std::string &value)
{
	std::string out;
	for (char ch : value)
	{
		switch (ch)
		{
		case '\\':
			out += "\\\\";
			break;
		case '"':
			out += "\\\"";
			break;
		case '\n':
			out += "\\n";
			break;
		case '\r':
			out += "\\r";
			break;
		case '\t':
			out += "\\t";
			break;
		default:
			out += ch;
		}
	}
	return out;
}

// The progress snapshots of a device run (ProgressTracker,
// src/runtime/progress.cpp:139-300): a running snapshot before the tree is
// launched and the final one after it.  Latest record in <run>.progress.json
// (or the configured path), history in the same name with .jsonl.
class ProgressTracker
{
  public:
	ProgressTracker(const SimulationConfig &config, int rank, int total_states,
					std::chrono::steady_clock::time_point start)
		: config_(config), rank_(rank), total_states_(total_states), start_(start), last_emit_(start)
	{
		if (enabled())
			path_ = latest_path().string();
	}

	const std::string &progress_path() const { return path_; }

	void replace_state(int evaluated_states, double prior_mass, const TreeStats &stats)
	{
		const int known = stats_.total_leaves;
		evaluated_ = evaluated_states;
		prior_mass_ = prior_mass;
		stats_ = stats;
		if (stats_.total_leaves == 0)
			stats_.total_leaves = known;
	}

	void maybe_emit(const std::string &message, bool force)
	{
		if (!enabled())
			return;
		const auto now = std::chrono::steady_clock::now();
		if (!force && std::chrono::duration<double>(now - last_emit_).count() < config_.progress.interval_seconds)
			return;
		const TerminationReason reason = simulation_cancellation_reason();
		write(reason == TerminationReason::none ? SimulationRunStatus::running : SimulationRunStatus::interrupted,
			  reason, message);
		last_emit_ = now;
	}

	void finish(SimulationRunStatus status, TerminationReason reason, const std::string &message)
	{
		if (enabled())
			write(status, reason, message);
	}

  private:
	bool enabled() const { return config_.progress.enabled && rank_ == 0; }

	std::filesystem::path latest_path() const
	{
		if (!config_.progress.output_path.empty())
			return config_.progress.output_path;
		return config_.report.output_directory / (run_name(config_) + ".progress.json");
	}

  public:
	// The record the tracker writes now (ProgressTracker::snapshot,
	// src/runtime/progress.cpp:217-261).
	ProgressSnapshot snapshot(SimulationRunStatus status, TerminationReason reason, const std::string &message) const
	{
		ProgressSnapshot snap;
		snap.status = status;
		snap.reason = reason;
		snap.total_states = total_states_;
		snap.evaluated_states = evaluated_;
		snap.state_coverage_fraction =
			total_states_ == 0 ? 0.0 : static_cast<double>(evaluated_) / static_cast<double>(total_states_);
		snap.evaluated_prior_mass = prior_mass_;
		snap.stats = stats_;
		snap.timings.total_seconds = seconds_since(start_);
		snap.message = message;
		return snap;
	}

  private:
	void write(SimulationRunStatus status, TerminationReason reason, const std::string &message) const
	{
		const ProgressSnapshot snap = snapshot(status, reason, message);
		const double elapsed = snap.timings.total_seconds;
		const double coverage = snap.state_coverage_fraction;
		const TreeStats &st = snap.stats;
		std::ostringstream body;
		body << std::setprecision(17) << "{\"status\":\"" << status_name(snap.status)
			 << "\",\"termination_reason\":\"" << reason_name(snap.reason) << "\",\"total_states\":" << snap.total_states
			 << ",\"evaluated_states\":" << snap.evaluated_states << ",\"state_coverage_fraction\":" << coverage
			 << ",\"evaluated_prior_mass\":" << snap.evaluated_prior_mass << ",\"stats\":{\"total_leaves\":" << st.total_leaves
			 << ",\"correct_probability\":" << st.correct_probability
			 << ",\"incorrect_probability\":" << st.incorrect_probability
			 << ",\"false_positive_probability\":" << st.false_positive_probability
			 << ",\"false_negative_probability\":" << st.false_negative_probability
			 << ",\"unclassified_probability\":" << st.unclassified_probability
			 << ",\"expected_stages\":" << st.expected_stages << ",\"expected_tests\":" << st.expected_tests
			 << "},\"timings\":{\"setup_seconds\":0,\"tree_build_seconds\":0,\"evaluation_seconds\":0,"
			 << "\"total_seconds\":" << elapsed << "},\"message\":\"" << json_escape(snap.message) << "\"}";
		const std::filesystem::path latest = latest_path();
		if (!latest.parent_path().empty())
			std::filesystem::create_directories(latest.parent_path());
		const std::filesystem::path tmp = latest.string() + ".tmp";
		{
			std::ofstream out(tmp, std::ios::trunc);
			out << body.str() << '\n';
		}
		std::filesystem::rename(tmp, latest);
		if (config_.progress.write_jsonl)
		{
			std::filesystem::path history = latest;
			history.replace_extension(".jsonl");
			std::ofstream out(history, std::ios::app);
			out << body.str() << '\n';
		}
		if (config_.progress.print_stderr)
		{
			std::cerr << "bgt progress: status=" << status_name(status) << " evaluated=" << evaluated_ << '/'
					  << total_states_ << " coverage=" << coverage << " prior_mass=" << prior_mass_
					  << " elapsed=" << elapsed << "s";
			if (!message.empty())
				std::cerr << " " << message;
			std::cerr << '\n';
		}
	}

	const SimulationConfig &config_;
	int rank_;
	int total_states_;
	std::chrono::steady_clock::time_point start_, last_emit_;
	int evaluated_ = 0;
	double prior_mass_ = 0.0;
	TreeStats stats_{};
	std::string path_;
};

} // namespace detail

inline bool cuda_available() { return bgt_cuda_provider_available() != 0; }

namespace detail
{

// resolve_selector (src/runtime/simulation_helpers.cpp:40-45).
inline SelectorType resolve_selector(SelectorType selector, int variants)
{
	if (selector != SelectorType::auto_select)
		return selector;
	return variants == 1 ? SelectorType::op_bha : SelectorType::op_bbpa;
}

// Runtime::make_kernel_spec (src/runtime/simulation_runner.cpp:166-179).
inline KernelSpec kernel_spec(const SimulationConfig &config)
{
	KernelSpec spec;
	spec.provider = config.options.provider;
	spec.subjects = config.subjects;
	spec.variants = config.variants;
	spec.dilution = uses_dilution(config.lattice_type) ? DilutionMode::dilution : DilutionMode::non_dilution;
	spec.selector = resolve_selector(config.options.selector, config.variants);
	spec.compile_options = config.options.compile_options;
	spec.precision = config.options.compile_options.posterior_precision;
	spec.accumulator_precision = config.options.compile_options.accumulator_precision;
	return spec;
}

} // namespace detail

// bgt::run_simulation for local trees on the device (Runtime::run_simulation,
// src/runtime/simulation_runner.cpp:181-262, through CudaProvider::run):
// validation, cancellation before evaluation, progress snapshots, the run
// and the CSV report.
inline SimulationResult run_simulation(const SimulationConfig &config)
{
	const auto total_start = std::chrono::steady_clock::now();
	const SimulationOptions &o = config.options;
	const int atoms = config.subjects * config.variants;
	if (config.subjects <= 0 || config.variants <= 0 || o.search_depth < 0)
		throw Error(StatusCode::invalid_argument, "invalid simulation dimensions.");
	if (config.workload_granularity <= 0)
		throw Error(StatusCode::invalid_argument, "workload_granularity must be positive.");
	if (config.progress.interval_seconds <= 0.0)
		throw Error(StatusCode::invalid_argument, "progress interval must be positive.");
	if (config.prior.size() != static_cast<std::size_t>(atoms))
		throw Error(StatusCode::invalid_argument, "prior length must equal subjects * variants.");
	if (config.evaluation_prior && config.evaluation_prior->size() != static_cast<std::size_t>(atoms))
		throw Error(StatusCode::invalid_argument, "evaluation_prior length must equal subjects * variants.");
	if (config.lattice_type == LatticeType::distributed_non_dilution ||
		config.lattice_type == LatticeType::distributed_dilution)
		throw Error(StatusCode::invalid_argument, "local_tree requires a replicated lattice.");
	if (config.mode != SimulationMode::local_tree)
		throw Error(StatusCode::unsupported,
					"parallel simulation modes need the MPI backend; the GB300 provider serves local_tree on one GPU.");
	if (o.provider == Provider::cpu)
		throw Error(StatusCode::unsupported, "the CPU provider is the reference library's.");
	const bool dil = detail::uses_dilution(config.lattice_type);
	if (dil && (config.dilution.alpha <= 0.0 || config.dilution.h <= 0.0))
		throw Error(StatusCode::invalid_argument, "dilution parameters must be positive.");
	if (config.test_accuracy && dil)
		throw Error(StatusCode::invalid_argument, "test accuracy applies to non-dilution models.");

	if (!config.options.compile_options.enable_cuda && o.provider == Provider::cuda)
		throw Error(StatusCode::unsupported, "CUDA provider requested, but CUDA is disabled in compile options.");
	SimulationResult r;
	r.kernel = detail::kernel_spec(config);
	r.mode = config.mode;
	r.total_states = atoms >= 31 ? 0 : (1 << atoms);
	detail::ProgressTracker progress(config, r.rank, r.total_states, total_start);
	const auto eval_start = std::chrono::steady_clock::now();
	if (simulation_cancellation_requested())
	{
		r.status = SimulationRunStatus::interrupted;
		r.termination_reason = simulation_cancellation_reason();
		r.progress_path = progress.progress_path();
		r.timings.total_seconds = detail::seconds_since(total_start);
		progress.finish(r.status, r.termination_reason, "cancelled before evaluation started");
		r.report_path = write_report_if_requested(config, r);
		return r;
	}
	if (!cuda_available())
		throw Error(StatusCode::cuda_error, "CUDA provider requested, but no CUDA device is available.");
	progress.maybe_emit("starting CUDA evaluation", true);
	DilutionTable table;
	if (dil)
		table = DilutionTable(config.subjects, config.dilution.alpha, config.dilution.h);
	bgt_tree_stats st{};
	if (config.test_accuracy)
		detail::check(bgt_gpu_tree_run_accuracy(config.subjects, config.variants, config.prior.data(), o.search_depth,
												o.threshold_up, o.threshold_lo, o.branch_threshold,
												static_cast<int>(o.selector), config.test_accuracy->sensitivity,
												config.test_accuracy->specificity, &st));
	else
		detail::check(bgt_cuda_provider_run(dil ? 1 : 0, config.subjects, config.variants, config.prior.data(),
											o.search_depth, o.threshold_up, o.threshold_lo, o.branch_threshold,
											static_cast<int>(o.selector), dil ? table.rows() : nullptr, &st));
	r.stats = TreeStats{st.total_leaves,
						st.correct_probability,
						st.incorrect_probability,
						st.false_positive_probability,
						st.false_negative_probability,
						st.unclassified_probability,
						st.expected_stages,
						st.expected_tests};
	r.provider = Provider::cuda;
	r.kernel.provider = Provider::cuda;
	r.evaluated_states = r.total_states;
	r.evaluated_prior_mass = 1.0;
	progress.replace_state(r.evaluated_states, r.evaluated_prior_mass, r.stats);
	r.timings.evaluation_seconds = detail::seconds_since(eval_start);
	r.timings.total_seconds = detail::seconds_since(total_start);
	r.progress_path = progress.progress_path();
	progress.finish(r.status, r.termination_reason, "completed");
	r.report_path = write_report_if_requested(config, r);
	return r;
}

// bgt::CudaProvider (include/bgt/runtime.hpp:50-56): one tree simulation
// through bgt_cuda_provider_run (CudaProvider::run, src/runtime/providers.cpp:73-133).
class CudaProvider
{
  public:
	bool available() const { return cuda_available(); }
	// `accuracy` (an extension) replaces the non-dilution likelihood.
	TreeStats run(LatticeType type, int subjects, int variants, std::span<const host_probability_t> prior,
				  const SimulationOptions &options, const DilutionTable *dilution,
				  const TestAccuracy *accuracy = nullptr) const
	{
		if (prior.size() != static_cast<std::size_t>(subjects) * static_cast<std::size_t>(variants))
			throw Error(StatusCode::invalid_argument, "prior length must equal subjects * variants.");
		const bool dil = detail::uses_dilution(type);
		if (dil && dilution == nullptr)
			throw Error(StatusCode::invalid_argument, "dilution table is required for dilution models.");
		if (dil && accuracy != nullptr)
			throw Error(StatusCode::invalid_argument, "test accuracy applies to non-dilution models.");
		bgt_tree_stats st{};
		if (accuracy != nullptr)
			detail::check(bgt_gpu_tree_run_accuracy(subjects, variants, prior.data(), options.search_depth,
													options.threshold_up, options.threshold_lo,
													options.branch_threshold, static_cast<int>(options.selector),
													accuracy->sensitivity, accuracy->specificity, &st));
		else
			detail::check(bgt_cuda_provider_run(dil ? 1 : 0, subjects, variants, prior.data(), options.search_depth,
												options.threshold_up, options.threshold_lo, options.branch_threshold,
												static_cast<int>(options.selector),
												dil ? const_cast<host_probability_t **>(dilution->rows()) : nullptr,
												&st));
		return TreeStats{st.total_leaves,
						 st.correct_probability,
						 st.incorrect_probability,
						 st.false_positive_probability,
						 st.false_negative_probability,
						 st.unclassified_probability,
						 st.expected_stages,
						 st.expected_tests};
	}
};

// ---- Logging settings (include/bgt/logging.hpp:11-52, behaviour of
// src/runtime/logging.cpp): a process-wide configuration, the environment
// variables BGT_LOG_LEVEL / BGT_LOG_SUBSYS / BGT_LOG_FILE / BGT_LOG_RANKS /
// BGT_LOG_COLOR / BGT_PERF_LEVEL applied on the first read.  This process is
// one rank, so the rank filter never drops a message.
enum class LogLevel
{
	off = 0,
	fatal = 1,
	error = 2,
	warn = 3,
	info = 4,
	debug = 5,
	trace = 6
};

enum class LogSubsystem
{
	core,
	model,
	tree,
	runtime,
	parallel,
	cuda,
	jit,
	perf
};

struct LogConfig
{
	LogLevel level = LogLevel::warn;
	std::vector<LogSubsystem> subsystems;
	std::vector<int> rank_filter;
	bool color = false;
	bool timestamps = true;
	std::filesystem::path file_path;
};

inline LogLevel parse_log_level(std::string_view value)
{
	std::string v(value);
	for (char &c : v)
		c = static_cast<char>(std::tolower(static_cast<unsigned char>(c)));
	const std::pair<const char *, LogLevel> names[] = {
		{"off", LogLevel::off},	  {"fatal", LogLevel::fatal}, {"error", LogLevel::error}, {"warn", LogLevel::warn},
		{"warning", LogLevel::warn}, {"info", LogLevel::info},	  {"debug", LogLevel::debug}, {"trace", LogLevel::trace}};
	for (const auto &[name, level] : names)
		if (v == name)
			return level;
	return LogLevel::warn;
}

inline LogSubsystem parse_log_subsystem(std::string_view value)
{
	std::string v(value);
	for (char &c : v)
		c = static_cast<char>(std::tolower(static_cast<unsigned char>(c)));
	const char *names[] = {"core", "model", "tree", "runtime", "parallel", "cuda", "jit", "perf"};
	for (int i = 0; i < 8; i++)
		if (v == names[i])
			return static_cast<LogSubsystem>(i);
	return LogSubsystem::runtime;
}

inline const char *log_level_name(LogLevel level)
{
	const char *names[] = {"OFF", "FATAL", "ERROR", "WARN", "INFO", "DEBUG", "TRACE"};
	const int i = static_cast<int>(level);
	return i >= 0 && i < 7 ? names[i] : "UNKNOWN";
}

inline const char *log_subsystem_name(LogSubsystem subsystem)
{
	const char *names[] = {"core", "model", "tree", "runtime", "parallel", "cuda", "jit", "perf"};
	const int i = static_cast<int>(subsystem);
	return i >= 0 && i < 8 ? names[i] : "unknown";
}

namespace detail
{

struct LogState
{
	std::mutex mutex;
	LogConfig config;
	bool env_applied = false;
};

inline LogState &log_state()
{
	static LogState state;
	return state;
}

inline std::vector<std::string> split_list(const std::string &value)
{
	std::vector<std::string> parts;
	std::string cur;
	for (char c : value)
	{
		if (c == ',')
		{
			if (!cur.empty())
				parts.push_back(cur);
			cur.clear();
		}
		else
			cur.push_back(c);
	}
	if (!cur.empty())
		parts.push_back(cur);
	return parts;
}

// Caller holds the state's mutex.
inline void apply_log_environment(LogState &st)
{
	if (st.env_applied)
		return;
	st.env_applied = true;
	if (const char *v = std::getenv("BGT_LOG_LEVEL"))
		st.config.level = parse_log_level(v);
	if (const char *v = std::getenv("BGT_LOG_SUBSYS"))
	{
		st.config.subsystems.clear();
		for (const std::string &p : split_list(v))
			st.config.subsystems.push_back(parse_log_subsystem(p));
	}
	if (const char *v = std::getenv("BGT_LOG_FILE"))
		st.config.file_path = v;
	if (const char *v = std::getenv("BGT_LOG_RANKS"))
	{
		st.config.rank_filter.clear();
		for (const std::string &p : split_list(v))
			st.config.rank_filter.push_back(std::stoi(p));
	}
	if (const char *v = std::getenv("BGT_LOG_COLOR"))
	{
		const std::string c = v;
		st.config.color = c == "1" || c == "true" || c == "on" || c == "TRUE" || c == "ON";
	}
	if (const char *v = std::getenv("BGT_PERF_LEVEL"))
	{
		const LogLevel perf = parse_log_level(v);
		if (static_cast<int>(perf) > static_cast<int>(st.config.level))
			st.config.level = perf;
		bool has = false;
		for (LogSubsystem s : st.config.subsystems)
			has = has || s == LogSubsystem::perf;
		if (!has)
			st.config.subsystems.push_back(LogSubsystem::perf);
	}
}

} // namespace detail

inline void set_log_config(LogConfig config)
{
	auto &st = detail::log_state();
	std::lock_guard<std::mutex> lock(st.mutex);
	st.config = std::move(config);
}

inline LogConfig get_log_config()
{
	auto &st = detail::log_state();
	std::lock_guard<std::mutex> lock(st.mutex);
	detail::apply_log_environment(st);
	return st.config;
}

inline void set_log_level(LogLevel level)
{
	auto &st = detail::log_state();
	std::lock_guard<std::mutex> lock(st.mutex);
	st.config.level = level;
}

inline bool log_enabled(LogLevel level, LogSubsystem subsystem)
{
	auto &st = detail::log_state();
	std::lock_guard<std::mutex> lock(st.mutex);
	detail::apply_log_environment(st);
	if (st.config.level == LogLevel::off || level == LogLevel::off)
		return false;
	if (static_cast<int>(level) > static_cast<int>(st.config.level))
		return false;
	if (st.config.subsystems.empty())
		return true;
	for (LogSubsystem s : st.config.subsystems)
		if (s == subsystem)
			return true;
	return false;
}

// Device-memory budget of lattice handles (bgt_gpu_set_memory_limit): an
// allocation past it throws Error(cuda_error) before the device is asked;
// 0 removes the limit.
inline void set_memory_limit(std::uint64_t bytes) { detail::check(bgt_gpu_set_memory_limit(bytes)); }
inline std::uint64_t memory_in_use()
{
	uint64_t bytes = 0;
	detail::check(bgt_gpu_memory_in_use(&bytes));
	return bytes;
}

// The CPU provider is always available, as in the reference; this package
// runs only the device path.
inline std::vector<Provider> available_providers()
{
	std::vector<Provider> out{Provider::cpu};
	if (cuda_available())
		out.push_back(Provider::cuda);
	return out;
}

// bgt::Runtime (include/bgt/runtime.hpp:58-74) without run-time compilation:
// the kernels are built ahead of time for sm_103a, so the JIT cache is empty.
class Runtime
{
  public:
	Runtime() = default;
	explicit Runtime(std::filesystem::path cache_directory) : cache_directory_(std::move(cache_directory)) {}

	std::vector<Provider> available_providers() const { return bgt::available_providers(); }
	JitCacheInfo jit_cache_info() const
	{
		JitCacheInfo info;
		info.disk_cache_directory = cache_directory_.string();
		return info;
	}
	void clear_jit_cache() {}
	KernelSpec make_kernel_spec(const SimulationConfig &config) const { return detail::kernel_spec(config); }
	SimulationResult run_simulation(const SimulationConfig &config) { return bgt::run_simulation(config); }

  private:
	std::filesystem::path cache_directory_;
};

inline JitCacheInfo jit_cache_info() { return Runtime{}.jit_cache_info(); }
inline void clear_jit_cache() {}

} // namespace bgt
