// `synchro` command-line drop-in (the reference's app/main.cpp:10-81 with
// app/args.hpp:51-78 and app/io.hpp:95-142), driving the GPU library through
// its C ABI.  Same flags, input format and output line; no JIT step: one
// binary serves every (n, k).
#include <unistd.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/synchrowords.h"

namespace {

enum Level { ERROR = 0, WARNING = 1, INFO = 2, VERBOSE = 3, DEBUG = 4 };
int g_level = INFO;

// [hh:mm:ss.mmm] [LEVEL] prefix (synchrolib/utils/logger.hpp:35-44).
void log(int level, const std::string& msg) {
  if (level > g_level) return;
  static const char* names[] = {"ERROR", "WARNING", "INFO", "VERBOSE", "DEBUG"};
  auto now = std::chrono::system_clock::now();
  auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(now.time_since_epoch()).count() % 1000;
  std::time_t t = std::chrono::system_clock::to_time_t(now);
  std::tm bt{};
  localtime_r(&t, &bt);
  char buf[32];
  std::strftime(buf, sizeof buf, "%H:%M:%S", &bt);
  std::printf("[%s.%03d] [%s] %s\n", buf, (int)ms, names[level], msg.c_str());
  std::fflush(stdout);
}

[[noreturn]] void die(const std::string& msg, int code) {
  log(ERROR, msg);
  std::exit(code);
}

struct Args {
  std::string input, config, output, suffix, model;
  bool has_output = false, verbose = false, quiet = false, debug = false, cont = false;
};

void usage() {
  std::printf(
      "Find synchronizing word of an automaton\n"
      "Usage:\n  synchro [OPTION...]\n\n"
      "  -f, --file arg          Path to the input file\n"
      "  -c, --config arg        Path to the config file\n"
      "  -o, --output arg        Path to the output file\n"
      "  -b, --build-suffix arg  Suffix of the build folder (accepted, unused: no JIT) (default: )\n"
      "      --continue          Do not overwrite the output file and run algorithms\n"
      "                          only for remaining automata\n"
      "  -v, --verbose           Verbose output\n"
      "  -q, --quiet             Quiet output (only warnings and errors)\n"
      "  -d, --debug             Debug output (all messages and timers)\n"
      "  -m, --model arg         Distance model for LearnedBeam (default: the packaged\n"
      "                          ../models/distance_mlp.f32 beside this program, if present)\n"
      "  -h, --help              Print usage\n");
}

Args parse(int argc, char** argv) {
  Args a;
  bool have_f = false, have_c = false;
  for (int i = 1; i < argc; ++i) {
    std::string s = argv[i];
    auto value = [&](const char* name) -> std::string {
      auto eq = s.find('=');
      if (s.rfind("--", 0) == 0 && eq != std::string::npos) return s.substr(eq + 1);
      if (i + 1 >= argc) die(std::string("Option '") + name + "' is missing an argument", 1);
      return argv[++i];
    };
    if (s == "-h" || s == "--help") {
      usage();
      std::exit(0);
    } else if (s == "-f" || s.rfind("--file", 0) == 0) {
      a.input = value("file");
      have_f = true;
    } else if (s == "-c" || s.rfind("--config", 0) == 0) {
      a.config = value("config");
      have_c = true;
    } else if (s == "-o" || s.rfind("--output", 0) == 0) {
      a.output = value("output");
      a.has_output = true;
    } else if (s == "-b" || s.rfind("--build-suffix", 0) == 0) {
      a.suffix = value("build-suffix");
    } else if (s == "-m" || s.rfind("--model", 0) == 0) {
      a.model = value("model");
    } else if (s == "--continue") {
      a.cont = true;
    } else if (s == "-v" || s == "--verbose") {
      a.verbose = true;
    } else if (s == "-q" || s == "--quiet") {
      a.quiet = true;
    } else if (s == "-d" || s == "--debug") {
      a.debug = true;
    } else {
      die("Option '" + s + "' does not exist", 1);
    }
  }
  if (!have_f) die("Required argument \xe2\x80\x98" "file" "\xe2\x80\x99 not found", 1);
  if (!have_c) die("Required argument \xe2\x80\x98" "config" "\xe2\x80\x99 not found", 1);
  if ((int)a.verbose + (int)a.quiet + (int)a.debug > 1)
    die("Only one of [--verbose, --quiet, --debug] can be enabled at one time", 1);
  if (a.cont && !a.has_output) die("--continue can be enabled only if an output file is specified", 1);
  return a;
}

struct Encoded {
  uint32_t n, k;
  std::vector<uint32_t> delta;
};

// app/io.hpp:136-159 — "K N" then N*K transitions, many automata per file.
std::vector<Encoded> read_automata(const std::string& path) {
  std::ifstream in(path);
  std::vector<Encoded> out;
  long long K, N;
  while (in >> K >> N) {
    if (N <= 0 || K <= 0) die("N and K must be greater than 0", 3);
    Encoded e{(uint32_t)N, (uint32_t)K, {}};
    e.delta.resize((size_t)N * K);
    for (size_t i = 0; i < e.delta.size(); ++i) {
      long long x;
      if (!(in >> x)) die("Expected " + std::to_string(N * K) + " integers, found " + std::to_string(i), 3);
      if (x < 0 || x >= N)
        die("Expected integer in range [0, " + std::to_string(N - 1) + "], found " + std::to_string(x), 3);
      e.delta[i] = (uint32_t)x;
    }
    out.push_back(std::move(e));
  }
  log(INFO, "Read " + std::to_string(out.size()) + " automata");
  return out;
}

size_t count_nonempty_lines(const std::string& path) {
  std::ifstream in(path);
  size_t c = 0;
  std::string s;
  while (std::getline(in, s))
    if (s.find_first_not_of(" \t\r\n\v\f") != std::string::npos) ++c;
  return c;
}

}  // namespace

int main(int argc, char** argv) {
  Args args = parse(argc, argv);
  if (args.verbose) g_level = VERBOSE;
  else if (args.quiet) g_level = WARNING;
  else if (args.debug) g_level = DEBUG;

  auto auts = read_automata(args.input);
  std::string config;
  {
    std::ifstream in(args.config);
    if (!in) die("cannot open config " + args.config, 2);
    std::stringstream ss;
    ss << in.rdbuf();
    config = ss.str();
  }
  size_t skip = 0;
  std::FILE* out = nullptr;
  if (args.has_output) {
    if (args.cont) {
      skip = count_nonempty_lines(args.output);
      out = std::fopen(args.output.c_str(), "a");
    } else {
      out = std::fopen(args.output.c_str(), "w");
    }
    if (!out) die("Error while opening the output file", 1);
  }
  if (skip) log(INFO, "Skipping " + std::to_string(skip) + " automata");

  sw_context* ctx = nullptr;
  if (sw_context_create(0, &ctx) != SW_OK) die(std::string("GPU unavailable: ") + sw_last_error(), 4);
  {
    // the distance model LearnedBeam ranks by: --model, else the packaged one
    std::string path = args.model;
    if (path.empty()) {
      char exe[4096];
      const ssize_t len = readlink("/proc/self/exe", exe, sizeof exe - 1);
      if (len > 0) {
        exe[len] = 0;
        std::string dir(exe);
        dir = dir.substr(0, dir.rfind('/'));
        path = dir + "/../models/distance_mlp.f32";
      }
    }
    std::ifstream mf(path, std::ios::binary);
    if (mf) {
      std::vector<float> params(SW_MLP_PARAMS);
      mf.read(reinterpret_cast<char*>(params.data()), sizeof(float) * params.size());
      if (mf.gcount() != (std::streamsize)(sizeof(float) * params.size()))
        die("Model file " + path + " does not hold " + std::to_string(SW_MLP_PARAMS) + " floats", 1);
      if (sw_context_set_model(ctx, params.data(), SW_MLP_PARAMS) != SW_OK) die(sw_last_error(), 4);
    } else if (!args.model.empty()) {
      die("Error while opening the model file", 1);
    }
  }

  size_t index = 0;
  for (const auto& a : auts) {
    if (index < skip) {
      ++index;
      continue;
    }
    sw_plan plan;
    if (sw_plan_from_json(config.c_str(), a.n, a.k, &plan) != SW_OK)
      die(std::string("Config exception: ") + sw_last_error(), 4);
    std::vector<uint32_t> word(1u << 20);
    sw_result r{};
    r.word = word.data();
    r.word_capacity = (uint32_t)word.size();
    int rc = sw_solve(ctx, a.delta.data(), a.n, a.k, &plan, &r);
    if (rc != SW_OK) die(sw_last_error(), 4);
    if (r.non_synchro) {
      log(INFO, "NON SYNCHRO");
    } else {
      log(INFO, "Minimum synchronizing word length: [" + std::to_string(r.mlsw_lower_bound) + ", " +
                    std::to_string(r.mlsw_upper_bound) + "]");
    }
    if (out) {
      // app/io.hpp:176-224
      std::fprintf(out, "%zu: ", index);
      if (r.non_synchro) {
        std::fprintf(out, "NON SYNCHRO\n");
      } else {
        std::fprintf(out, "[%llu, %llu] (", (unsigned long long)r.mlsw_lower_bound,
                     (unsigned long long)r.mlsw_upper_bound);
        for (uint32_t i = 0; i < r.n_runs; ++i)
          std::fprintf(out, "%s(%s, %llu)", i ? ", " : "", r.runs[i].name, (unsigned long long)r.runs[i].ms);
        std::fprintf(out, ")");
        if (r.has_word) {
          std::fprintf(out, " {");
          for (uint32_t i = 0; i < r.word_len; ++i) std::fprintf(out, "%s%u", i ? " " : "", word[i]);
          std::fprintf(out, "}");
        }
        std::fprintf(out, "\n");
      }
      std::fflush(out);
    } else if (r.has_word) {
      log(INFO, "Found synchronizing word of length " + std::to_string(r.word_len) +
                    " (use the -o flag to save it)");
    }
    ++index;
  }
  if (out) std::fclose(out);
  sw_context_destroy(ctx);
  return 0;
}
