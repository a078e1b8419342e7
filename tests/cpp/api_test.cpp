// The C++20 host API (include/bgt_gb300/bgt.hpp) against the reference's own
// C++ pins: tests/cpp/unit/lattice_api_test.cpp:63-99 (public order, upset
// masses, selections, update, classification, multinomial BBPA = brute
// force), tests/cpp/unit/dilution_test.cpp:11-13 (table rows) and the
// single-subject TreeStats golden of tests/cpp/support/assertions.hpp:80-92,
// plus the run report and progress files of run_simulation
// (src/runtime/reporting.cpp:10-45).  argv[1]: a scratch directory.
// Exit status 0 = pass; prints "skip" without a device.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <filesystem>
#include <fstream>
#include <map>
#include <string>
#include <vector>

#include "bgt_gb300/bgt.hpp"

namespace
{

int failures = 0;

void expect_near(double got, double want, double tol, const char *what)
{
	if (!(std::fabs(got - want) <= tol))
	{
		std::printf("FAIL %s: got %.17g want %.17g\n", what, got, want);
		failures++;
	}
}

void expect_equal(long long got, long long want, const char *what)
{
	if (got != want)
	{
		std::printf("FAIL %s: got %lld want %lld\n", what, got, want);
		failures++;
	}
}

template <typename F>
void expect_error(F &&f, bgt::StatusCode code, const char *what)
{
	try
	{
		f();
		std::printf("FAIL %s: no error\n", what);
		failures++;
	}
	catch (const bgt::Error &e)
	{
		if (e.code() != code)
		{
			std::printf("FAIL %s: status %d\n", what, static_cast<int>(e.code()));
			failures++;
		}
	}
}

// Exhaustive BBPA for a k-variant lattice: for each experiment, the masses of
// the 2^k response buckets (bit v set when the pool holds a positive of
// variant v) and the score sum |mass - 1/2^k|; lowest experiment on ties.
bgt::state_t brute_force_bbpa(const bgt::Lattice &lat, int n, int k)
{
	const int states = 1 << (n * k);
	std::vector<double> post(static_cast<std::size_t>(states));
	for (int s = 0; s < states; s++)
		post[static_cast<std::size_t>(s)] = lat.posterior_probability(static_cast<bgt::state_t>(s));
	double best = 1e300;
	bgt::state_t best_e = 0;
	for (int e = 0; e < (1 << n); e++)
	{
		std::vector<double> mass(static_cast<std::size_t>(1) << k, 0.0);
		for (int s = 0; s < states; s++)
		{
			int r = 0;
			for (int v = 0; v < k; v++)
				if ((e & ~((s >> (n * v)) & ((1 << n) - 1))) != 0)
					r |= 1 << v;
			mass[static_cast<std::size_t>(r)] += post[static_cast<std::size_t>(s)];
		}
		double score = 0.0;
		for (double m : mass)
			score += std::fabs(m - 1.0 / static_cast<double>(mass.size()));
		if (score < best)
		{
			best = score;
			best_e = static_cast<bgt::state_t>(e);
		}
	}
	return best_e;
}

std::map<std::string, std::string> read_report(const std::filesystem::path &path)
{
	std::map<std::string, std::string> rows;
	std::ifstream in(path);
	std::string line;
	std::getline(in, line);
	if (line != "field,value")
	{
		std::printf("FAIL report header: %s\n", line.c_str());
		failures++;
	}
	while (std::getline(in, line))
	{
		const auto comma = line.find(',');
		rows[line.substr(0, comma)] = line.substr(comma + 1);
	}
	return rows;
}

void expect_field(const std::map<std::string, std::string> &rows, const char *key, const char *want)
{
	const auto it = rows.find(key);
	if (it == rows.end() || it->second != want)
	{
		std::printf("FAIL report %s: got '%s' want '%s'\n", key, it == rows.end() ? "(missing)" : it->second.c_str(),
					want);
		failures++;
	}
}

} // namespace

int main(int argc, char **argv)
{
	if (!bgt::cuda_available())
	{
		std::printf("skip\n");
		return 0;
	}
	const std::vector<double> prior{0.2, 0.4};
	bgt::Lattice lattice(bgt::LatticeType::replicated_non_dilution, 2, prior);
	expect_near(lattice.posterior_probability(0), 0.08, 1e-12, "prior state 0");
	expect_near(lattice.posterior_probability(1), 0.12, 1e-12, "prior state 1");
	expect_near(lattice.posterior_probability(2), 0.32, 1e-12, "prior state 2");
	expect_near(lattice.posterior_probability(3), 0.48, 1e-12, "prior state 3");
	expect_near(lattice.upset_probability_mass(1), 0.60, 1e-12, "upset mass 1");
	expect_near(lattice.upset_probability_mass(2), 0.80, 1e-12, "upset mass 2");
	expect_near(lattice.upset_probability_mass(3), 0.48, 1e-12, "upset mass 3");
	expect_near(lattice.response_probability(1, 1, 3), 0.99, 1e-15, "response probability, contained");
	expect_near(lattice.response_probability(1, 1, 2), 0.01, 1e-15, "response probability, not contained");
	expect_near(lattice.response_probability(3, 0, 1), 0.99, 1e-15, "response probability, positive");
	{
		bgt::Lattice accurate(bgt::LatticeType::replicated_non_dilution, 2, prior);
		accurate.set_test_accuracy(0.95, 0.98);
		expect_near(accurate.response_probability(1, 1, 3), 0.98, 1e-15, "specificity, contained pool");
		expect_near(accurate.response_probability(1, 0, 2), 0.95, 1e-15, "sensitivity, pooled positive");
	}
	expect_equal(lattice.select_experiment(), 3, "auto selection");
	expect_equal(lattice.select_experiment(bgt::SelectorType::op_bha), 3, "Op-BHA selection");
	expect_equal(lattice.select_experiment(bgt::SelectorType::op_bbpa), 3, "Op-BBPA selection");
	{
		// tests/cpp/unit/lattice_api_test.cpp:75-79
		const std::vector<bgt::state_t> lookahead = lattice.select_experiments(2, bgt::SelectorType::op_bha);
		expect_equal(static_cast<long long>(lookahead.size()), 2, "k-lookahead size");
		expect_equal(lookahead[0], 3, "k-lookahead first experiment");
		expect_equal(lookahead[1], 2, "k-lookahead second experiment");
		expect_equal(lattice.select_experiments(1, bgt::SelectorType::op_bbpa)[0], 3, "selector BBPA k=1 experiment");
		bool threw = false;
		try
		{
			(void)lattice.select_experiments(2, bgt::SelectorType::op_bbpa);
		}
		catch (const std::invalid_argument &)
		{
			threw = true;
		}
		expect_equal(threw, 1, "Op-BBPA lookahead throws std::invalid_argument");
	}
	lattice.update(1, 1);
	const double den = 0.60 * 0.99 + 0.40 * 0.01;
	expect_near(lattice.posterior_probability(0), 0.08 * 0.01 / den, 1e-12, "posterior state 0");
	expect_near(lattice.posterior_probability(1), 0.12 * 0.99 / den, 1e-12, "posterior state 1");
	expect_near(lattice.posterior_probability(2), 0.32 * 0.01 / den, 1e-12, "posterior state 2");
	expect_near(lattice.posterior_probability(3), 0.48 * 0.99 / den, 1e-12, "posterior state 3");
	lattice.update_classification(0.01, 0.01);
	expect_equal(lattice.positive_classification_mask(), 0, "positive mask");
	expect_equal(lattice.negative_classification_mask(), 1, "negative mask");
	expect_equal(lattice.is_classified(), 0, "not classified");

	{
		// Logging settings round trip (tests/python/unit/test_public_api.py:36-53 of the reference).
		bgt::LogConfig config;
		config.level = bgt::LogLevel::debug;
		config.subsystems = {bgt::LogSubsystem::runtime};
		config.rank_filter = {0, 2};
		config.timestamps = false;
		bgt::set_log_config(config);
		const bgt::LogConfig got = bgt::get_log_config();
		expect_equal(got.level == bgt::LogLevel::debug, 1, "log level round trip");
		expect_equal(got.subsystems.size() == 1 && got.subsystems[0] == bgt::LogSubsystem::runtime, 1,
					 "log subsystems round trip");
		expect_equal(got.rank_filter.size() == 2 && got.rank_filter[1] == 2, 1, "log rank filter round trip");
		expect_equal(bgt::log_enabled(bgt::LogLevel::info, bgt::LogSubsystem::runtime), 1, "runtime info enabled");
		expect_equal(bgt::log_enabled(bgt::LogLevel::info, bgt::LogSubsystem::cuda), 0, "cuda filtered out");
		bgt::set_log_level(bgt::LogLevel::warn);
		expect_equal(bgt::get_log_config().level == bgt::LogLevel::warn, 1, "set_log_level");
		expect_equal(bgt::parse_log_level("Warning") == bgt::LogLevel::warn, 1, "parse warning");
		expect_equal(std::string(bgt::log_level_name(bgt::LogLevel::trace)) == "TRACE", 1, "level name");
		bgt::set_log_config(bgt::LogConfig{});
	}

	{
		// Allocation failure through the lattice budget: an Error, nothing leaked.
		const std::uint64_t used = bgt::memory_in_use();
		bgt::set_memory_limit(used + 4096);
		expect_error([&] { bgt::Lattice big(bgt::LatticeType::replicated_non_dilution, 18, std::vector<double>(18, 0.05)); },
					 bgt::StatusCode::cuda_error, "lattice over the memory budget");
		bgt::set_memory_limit(0);
		expect_equal(static_cast<long long>(bgt::memory_in_use()), static_cast<long long>(used),
					 "failed create released its memory");
	}

	const std::vector<double> multinomial_prior{0.11, 0.23, 0.31, 0.41, 0.17, 0.29};
	bgt::Lattice multinomial(bgt::LatticeType::replicated_non_dilution, 3, 2, multinomial_prior);
	expect_equal(multinomial.select_experiment(bgt::SelectorType::op_bbpa), brute_force_bbpa(multinomial, 3, 2),
				 "multinomial BBPA = brute force");
	{
		// std::invalid_argument, as the reference's model throws (src/kernels/cpu/bbpa.cpp:864-867).
		bool threw = false;
		try
		{
			(void)multinomial.select_experiment(bgt::SelectorType::op_bha);
		}
		catch (const std::invalid_argument &)
		{
			threw = true;
		}
		expect_equal(threw, 1, "Op-BHA with two variants throws std::invalid_argument");
	}

	const bgt::DilutionTable table(2, 0.99, 0.005);
	expect_near(table.at(1, 0), 0.99, 1e-12, "dilution row 1, 0 positives");
	expect_near(table.at(1, 1), 0.01, 1e-12, "dilution row 1, 1 positive");
	expect_near(table.at(2, 1), 1.0 - 0.99 / 1.005, 1e-12, "dilution row 2, 1 positive");
	bgt::Lattice dil(bgt::LatticeType::replicated_dilution, 2, prior);
	expect_error([&] { dil.update(1, 1, nullptr); }, bgt::StatusCode::invalid_argument, "dilution update without table");
	dil.update(3, 0, &table);
	double total = 0.0;
	for (bgt::state_t s = 0; s < 4; s++)
		total += dil.posterior_probability(s);
	expect_near(total, 1.0, 1e-12, "dilution posterior sums to 1");

	bgt::SimulationConfig cfg;
	cfg.subjects = 1;
	cfg.prior = {0.2};
	cfg.options.search_depth = 1;
	cfg.options.provider = bgt::Provider::cuda;
	const bgt::TreeStats st = bgt::run_simulation(cfg).stats;
	expect_equal(st.total_leaves, 2, "single-subject leaves");
	expect_near(st.correct_probability, 0.792, 1e-12, "single-subject correct");
	expect_near(st.incorrect_probability, 0.002, 1e-12, "single-subject incorrect");
	expect_near(st.false_positive_probability, 0.0, 1e-12, "single-subject false positive");
	expect_near(st.false_negative_probability, 0.002, 1e-12, "single-subject false negative");
	expect_near(st.unclassified_probability, 0.206, 1e-12, "single-subject unclassified");
	expect_near(st.expected_stages, 1.0, 1e-12, "single-subject expected stages");
	expect_near(st.expected_tests, 1.0, 1e-12, "single-subject expected tests");
	{
		bgt::SimulationConfig acc = cfg;
		acc.test_accuracy = bgt::TestAccuracy{0.95, 0.98};
		const bgt::TreeStats sa = bgt::run_simulation(acc).stats;
		expect_equal(sa.total_leaves, 2, "accuracy: leaves");
		expect_near(sa.correct_probability + sa.incorrect_probability + sa.unclassified_probability, 1.0, 1e-12,
					"accuracy: outcomes sum to 1");
		expect_equal(std::abs(sa.correct_probability - st.correct_probability) > 1e-6, 1,
					 "accuracy: the likelihood reached the tree");
		acc.lattice_type = bgt::LatticeType::replicated_dilution;
		expect_error([&] { bgt::run_simulation(acc); }, bgt::StatusCode::invalid_argument,
					 "accuracy on a dilution lattice");
	}

	// Reports and progress files.
	const std::filesystem::path dir =
		argc > 1 ? std::filesystem::path(argv[1]) : std::filesystem::temp_directory_path() / "bgt_api_test";
	cfg.report.write_csv = true;
	cfg.report.output_directory = dir;
	cfg.report.run_name = "single";
	cfg.progress.enabled = true;
	const bgt::SimulationResult res = bgt::run_simulation(cfg);
	expect_equal(res.report_path == (dir / "single.csv").string(), 1, "report path");
	const auto rows = read_report(res.report_path);
	expect_field(rows, "status", "completed");
	expect_field(rows, "is_partial", "false");
	expect_field(rows, "mode", "local_tree");
	expect_field(rows, "provider", "2");
	expect_field(rows, "total_states", "2");
	expect_field(rows, "evaluated_states", "2");
	expect_field(rows, "state_coverage_fraction", "1");
	expect_field(rows, "total_leaves", "2");
	expect_field(rows, "correct_probability", "0.792");
	expect_field(rows, "unclassified_probability", "0.206");
	expect_field(rows, "expected_tests", "1");
	expect_equal(std::filesystem::exists(dir / "single.progress.json"), 1, "progress file");
	expect_equal(std::filesystem::exists(dir / "single.progress.jsonl"), 1, "progress history");
	bgt::request_simulation_cancellation();
	cfg.report.run_name = "cancelled";
	const bgt::SimulationResult cancelled = bgt::run_simulation(cfg);
	bgt::clear_simulation_cancellation();
	expect_equal(cancelled.status == bgt::SimulationRunStatus::interrupted, 1, "cancelled status");
	expect_equal(cancelled.report_path == (dir / "cancelled.partial.csv").string(), 1, "partial report path");
	expect_field(read_report(cancelled.report_path), "termination_reason", "cancellation_requested");
	cfg.mode = bgt::SimulationMode::parallel_global_tree;
	expect_error([&] { bgt::run_simulation(cfg); }, bgt::StatusCode::unsupported, "parallel mode");
	cfg.mode = bgt::SimulationMode::local_tree;
	cfg.report.write_csv = false;
	cfg.progress.enabled = false;

	// Runtime, KernelSpec and CudaProvider (include/bgt/runtime.hpp:50-74).
	bgt::Runtime runtime;
	const auto providers = runtime.available_providers();
	expect_equal(providers.size() == 2 && providers[1] == bgt::Provider::cuda, 1, "providers cpu, cuda");
	expect_equal(runtime.jit_cache_info().jit_enabled, 0, "no run-time compilation");
	bgt::SimulationConfig dcfg = cfg;
	dcfg.lattice_type = bgt::LatticeType::replicated_dilution;
	dcfg.variants = 1;
	const bgt::KernelSpec spec = runtime.make_kernel_spec(dcfg);
	expect_equal(spec.dilution == bgt::DilutionMode::dilution, 1, "spec dilution");
	expect_equal(spec.selector == bgt::SelectorType::op_bha, 1, "auto resolves to Op-BHA for k = 1");
	expect_equal(bgt::KernelSpecHash{}(spec) == bgt::KernelSpecHash{}(runtime.make_kernel_spec(dcfg)), 1, "spec hash");
	const bgt::SimulationResult rr = runtime.run_simulation(cfg);
	expect_equal(rr.kernel.provider == bgt::Provider::cuda, 1, "result kernel provider");
	expect_near(rr.stats.correct_probability, 0.792, 1e-12, "runtime run correct");
	const std::vector<double> single{0.2};
	const bgt::TreeStats ps = bgt::CudaProvider{}.run(bgt::LatticeType::replicated_non_dilution, 1, 1, single,
													  cfg.options, nullptr);
	expect_equal(ps.total_leaves, 2, "provider leaves");
	expect_near(ps.unclassified_probability, 0.206, 1e-12, "provider unclassified");
	cfg.options.compile_options.enable_cuda = false;
	expect_error([&] { bgt::run_simulation(cfg); }, bgt::StatusCode::unsupported, "CUDA disabled in compile options");

	std::printf("%s (%d failures)\n", failures ? "FAIL" : "ok", failures);
	return failures ? 1 : 0;
}
