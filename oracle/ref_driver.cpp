// Test-infrastructure driver for the compiled reference (SynchroLib 1.1.0).
//
// This file is part of the oracle: only tests, the smoke check and the CPU
// baseline leg of bench.py may run what it builds, and only as a checker.
// It is compiled by oracle/build_ref.py together with the reference's own,
// unmodified sources (read where they lie); the product never links it.
//
// What it does: the reference's CLI (app/main.cpp:10-81) re-JIT-compiles the
// library for every (N, K) and then calls the plugin entry point
// `extern "C" void run(...)` (jit/jitmain.cpp:11-49).  build_ref.py replaces the
// JIT step by compiling the library once for a fixed (AUT_N, AUT_K, plan), and
// this main() takes the place of app/main.cpp: it reads automata in the
// reference's input format (app/io.hpp:136-159), calls run() for each, and
// writes the reference's output line (app/io.hpp:176-224).
//
// Extra flags (not in the reference CLI): -L <level> picks the log level
// (0 error .. 4 debug), and automata whose N or K differ from the compiled
// ones are reported as "SKIP".
#include <jitdefines.hpp>

#include <synchrolib/algorithm/algorithm.hpp>
#include <synchrolib/utils/logger.hpp>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

extern "C" void run(const std::string& aut_encoded,
                    const std::vector<std::string>& algorithms,
                    synchrolib::AlgoResult& result,
                    synchrolib::Logger::LogLevel log_level);

#ifndef REF_ALGORITHMS
#error "REF_ALGORITHMS must list the plan's algorithm names"
#endif

static std::vector<std::string> plan_algorithms() {
  std::vector<std::string> out;
  std::stringstream ss(REF_ALGORITHMS);
  std::string name;
  while (std::getline(ss, name, ',')) {
    if (!name.empty()) out.push_back(name);
  }
  return out;
}

int main(int argc, char** argv) {
  const char* in_path = nullptr;
  const char* out_path = nullptr;
  int level = 2;
  for (int i = 1; i < argc; ++i) {
    if (!std::strcmp(argv[i], "-f") && i + 1 < argc) in_path = argv[++i];
    else if (!std::strcmp(argv[i], "-o") && i + 1 < argc) out_path = argv[++i];
    else if (!std::strcmp(argv[i], "-L") && i + 1 < argc) level = std::atoi(argv[++i]);
    else {
      std::fprintf(stderr, "usage: %s -f input [-o output] [-L level]\n", argv[0]);
      return 1;
    }
  }
  if (!in_path) {
    std::fprintf(stderr, "missing -f input\n");
    return 1;
  }
  std::ifstream in(in_path);
  if (!in) {
    std::fprintf(stderr, "cannot open %s\n", in_path);
    return 3;
  }
  std::FILE* out = out_path ? std::fopen(out_path, "w") : stdout;
  if (!out) {
    std::fprintf(stderr, "cannot open %s\n", out_path);
    return 1;
  }
  // Logs go to stderr so that stdout carries only result lines.
  synchrolib::Logger::set_log_stream(&std::cerr);
  const auto algos = plan_algorithms();
  const auto log_level = static_cast<synchrolib::Logger::LogLevel>(level);

  unsigned k = 0, n = 0;
  size_t index = 0;
  while (in >> k >> n) {
    std::string enc;
    for (size_t i = 0; i < static_cast<size_t>(k) * n; ++i) {
      unsigned x;
      in >> x;
      if (!enc.empty()) enc.push_back(' ');
      enc += std::to_string(x);
    }
    if (n != AUT_N || k != AUT_K) {
      std::fprintf(out, "%zu: SKIP\n", index++);
      continue;
    }
    synchrolib::AlgoResult result;
    run(enc, algos, result, log_level);
    if (result.non_synchro) {
      std::fprintf(out, "%zu: NON SYNCHRO\n", index++);
      std::fflush(out);
      continue;
    }
    std::fprintf(out, "%zu: [%llu, %llu] (", index++,
                 (unsigned long long)result.mlsw_lower_bound,
                 (unsigned long long)result.mlsw_upper_bound);
    for (size_t i = 0; i < result.algorithms_run.size(); ++i) {
      std::fprintf(out, "%s(%s, %zu)", i ? ", " : "",
                   result.algorithms_run[i].name.c_str(),
                   result.algorithms_run[i].time);
    }
    std::fprintf(out, ")");
    if (result.word) {
      std::fprintf(out, " {");
      for (size_t i = 0; i < result.word->size(); ++i)
        std::fprintf(out, "%s%u", i ? " " : "", (*result.word)[i]);
      std::fprintf(out, "}");
    }
    std::fprintf(out, "\n");
    std::fflush(out);
  }
  if (out != stdout) std::fclose(out);
  return 0;
}
