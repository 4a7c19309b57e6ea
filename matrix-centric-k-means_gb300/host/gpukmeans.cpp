// gpukmeans — command-line front end with the reference's flags, input and
// output formats, stdout lines and exit codes (src/main.cu:16-155,
// src/include/utils.hpp:16-171), over the Kmeans class of kmeans.hpp.
//
//   -d/--n-dimensions  -n/--n-samples  -k/--n-clusters  -m/--maxiter   (required)
//   -b/--init random|plusplus  -f/--kernel linear|polynomial|sigmoid  -l/--level (required)
//   -o/--out-file (default None)  -i/--in-file (.csv or .svm; else seeded random data)
//   -r/--runs (default 1)  -s/--seed (default std::rand())  -t/--tolerance (default FLT_EPSILON)
//   -c/--check 0|1 (default 0)  -h/--help
// Extensions: -f gaussian with --sigma S; -p/--precision auto|fp32|bf16|bf16x3;
//   --csv-columns reference|plain (plain keeps column 0); --profile prints the
//   per-stage [PERFORMANCE] lines of the linear path after each run.
//
// Exit codes (src/include/utils.hpp:34-37): 1 bad or missing argument, 2 no
// CUDA device, 3 point index out of bounds, 4 invalid input file; a library
// error exits 1 with its message, as the reference's CHECK_* macros do.
// As in the reference, run 0 is a warm-up excluded from the averages, so a
// single run prints an average of 0/0.
#include <cerrno>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <memory>
#include <string>
#include <vector>

#include "input_parser.hpp"
#include "kmeans.hpp"

namespace {

constexpr int EXIT_ARGS = 1;
constexpr int EXIT_CUDA_DEV = 2;
constexpr int EXIT_INVALID_INFILE = 4;

const char* const BOLDBLUE = "\033[1m\033[34m";
const char* const CYAN = "\033[36m";
const char* const RESET = "\033[0m";

struct Opt {
  char short_name;
  const char* long_name;
  const char* help;
  bool takes_value;
};

const Opt OPTS[] = {
    {'h', "help", "Print usage", false},
    {'d', "n-dimensions", "Number of dimensions of a point", true},
    {'n', "n-samples", "Number of points", true},
    {'k', "n-clusters", "Number of clusters", true},
    {'m', "maxiter", "Maximum number of iterations", true},
    {'o', "out-file", "Output filename", true},
    {'i', "in-file", "Input filename", true},
    {'r', "runs", "Number of k-means runs", true},
    {'s', "seed", "Seed for centroids generator", true},
    {'t', "tolerance", "Tolerance to declare convergence", true},
    {'c', "check", "Whether or not to check convergence", true},
    {'b', "init", "Method to use to initialize centroids", true},
    {'f', "kernel", "kernel function", true},
    {'l', "level", "Optimization level", true},
    {'p', "precision", "auto | fp32 | bf16 | bf16x3 (extension; auto: bf16x3 for -f linear, fp32 otherwise)", true},
    {0, "sigma", "Gaussian kernel width (extension)", true},
    {0, "csv-columns", "reference | plain (extension)", true},
    {0, "profile", "print per-stage timings (extension)", false},
};

void usage() {
  std::cout << "gpukmeans is an implementation of the K-means algorithm that uses a GPU\n"
               "Usage:\n  gpukmeans [OPTION...]\n\n";
  for (const Opt& o : OPTS) {
    std::string s = o.short_name ? std::string("  -") + o.short_name + ", --" : std::string("      --");
    s += o.long_name;
    if (o.takes_value) s += " arg";
    std::printf("%-30s %s\n", s.c_str(), o.help);
  }
}

[[noreturn]] void die_arg(const std::string& name) {
  std::cerr << "Invalid or missing argument: " << name << std::endl;
  std::exit(EXIT_ARGS);
}

// cxxopts-style parsing: -x VALUE, -xVALUE, --name VALUE, --name=VALUE.
std::map<std::string, std::string> parse(int argc, char** argv) {
  std::map<std::string, std::string> v;
  for (int a = 1; a < argc; ++a) {
    std::string arg = argv[a];
    const Opt* opt = nullptr;
    std::string val;
    bool have_val = false;
    if (arg.size() > 2 && arg[0] == '-' && arg[1] == '-') {
      std::string name = arg.substr(2);
      const size_t eq = name.find('=');
      if (eq != std::string::npos) {
        val = name.substr(eq + 1);
        name = name.substr(0, eq);
        have_val = true;
      }
      for (const Opt& o : OPTS)
        if (name == o.long_name) opt = &o;
    } else if (arg.size() >= 2 && arg[0] == '-') {
      for (const Opt& o : OPTS)
        if (o.short_name && arg[1] == o.short_name) opt = &o;
      if (opt && arg.size() > 2) {
        val = arg.substr(2);
        have_val = true;
      }
    }
    if (!opt) {
      std::cerr << "Option '" << arg << "' does not exist" << std::endl;
      std::exit(EXIT_ARGS);
    }
    if (opt->takes_value && !have_val) {
      if (a + 1 >= argc) die_arg(opt->long_name);
      val = argv[++a];
    }
    v[opt->long_name] = opt->takes_value ? val : "1";
  }
  return v;
}

long long get_int(const std::map<std::string, std::string>& v, const char* name, const long long* def) {
  auto it = v.find(name);
  if (it == v.end()) {
    if (def) return *def;
    die_arg(name);
  }
  const char* s = it->second.c_str();
  char* end = nullptr;
  errno = 0;
  const long long x = std::strtoll(s, &end, 10);
  if (errno || end == s || *end != '\0') die_arg(name);
  return x;
}

float get_float(const std::map<std::string, std::string>& v, const char* name, float def) {
  auto it = v.find(name);
  if (it == v.end()) return def;
  const char* s = it->second.c_str();
  char* end = nullptr;
  const float x = std::strtof(s, &end);
  if (end == s || *end != '\0') die_arg(name);
  return x;
}

std::string get_str(const std::map<std::string, std::string>& v, const char* name, const char* def) {
  auto it = v.find(name);
  if (it == v.end()) {
    if (def) return def;
    die_arg(name);
  }
  return it->second;
}

}  // namespace

int main(int argc, char** argv) {
  const auto args = parse(argc, argv);
  if (args.count("help")) {
    usage();
    return 0;
  }
  const long long d_ = get_int(args, "n-dimensions", nullptr);
  const long long n_ = get_int(args, "n-samples", nullptr);
  const long long k_ = get_int(args, "n-clusters", nullptr);
  const long long maxiter_ = get_int(args, "maxiter", nullptr);
  const std::string out_file = get_str(args, "out-file", "None");
  const float tol = get_float(args, "tolerance", FLT_EPSILON);
  const long long one = 1, zero = 0;
  const long long runs_ = get_int(args, "runs", &one);
  const bool check_converged = get_int(args, "check", &zero) != 0;
  const std::string init_str = get_str(args, "init", nullptr);
  const std::string kernel_str = get_str(args, "kernel", nullptr);
  const int level = static_cast<int>(get_int(args, "level", nullptr));
  if (d_ <= 0 || d_ > 0xffffffffLL) die_arg("n-dimensions");
  if (n_ <= 0) die_arg("n-samples");
  if (k_ <= 0 || k_ > 0xffffffffLL) die_arg("n-clusters");
  if (maxiter_ <= 0) die_arg("maxiter");
  if (runs_ <= 0) die_arg("runs");
  const uint32_t d = static_cast<uint32_t>(d_), k = static_cast<uint32_t>(k_);
  const size_t n = static_cast<size_t>(n_);
  const uint64_t maxiter = static_cast<uint64_t>(maxiter_);
  const uint32_t runs = static_cast<uint32_t>(runs_);

  // seed: -s, else std::rand() (utils.hpp:140-146)
  const int seed = args.count("seed") ? static_cast<int>(get_int(args, "seed", nullptr)) : std::rand();

  std::unique_ptr<InputParser<float>> input;
  if (args.count("in-file")) {
    const std::string in_file = args.at("in-file");
    InputParser<float>::InputFormat format;
    if (in_file.find(".csv") != std::string::npos)
      format = InputParser<float>::InputFormat::CSV;
    else if (in_file.find(".svm") != std::string::npos)
      format = InputParser<float>::InputFormat::SVM;
    else {
      std::cerr << "Invalid input file" << std::endl;
      return EXIT_INVALID_INFILE;
    }
    std::ifstream f(in_file, std::ios::in | std::ios::binary);
    if (!f) {
      std::cerr << "Invalid input file" << std::endl;
      return EXIT_INVALID_INFILE;
    }
    const std::string cols = get_str(args, "csv-columns", "reference");
    if (cols != "reference" && cols != "plain") die_arg("csv-columns");
    input.reset(new InputParser<float>(f, static_cast<int>(d), n, format,
                                       cols == "plain" ? InputParser<float>::CsvColumns::plain
                                                       : InputParser<float>::CsvColumns::reference));
    if (!input->ok()) {
      std::cerr << "Invalid input file" << std::endl;
      return EXIT_INVALID_INFILE;
    }
  } else {
    input.reset(new InputParser<float>(seed, static_cast<int>(d), n));
  }

  // extension argument: validated with the others, before the device check
  const std::string prec_str = get_str(args, "precision", "auto");
  Kmeans::Precision precision;
  if (prec_str == "auto") precision = Kmeans::Precision::automatic;
  else if (prec_str == "fp32") precision = Kmeans::Precision::fp32;
  else if (prec_str == "bf16") precision = Kmeans::Precision::bf16;
  else if (prec_str == "bf16x3") precision = Kmeans::Precision::bf16x3;
  else die_arg("precision");

  if (km_device_count() == 0) {
    std::cerr << "There are no available device(s) that support CUDA" << std::endl;
    return EXIT_CUDA_DEV;
  }

  std::printf("%s", BOLDBLUE);
  Kmeans::InitMethod init_method;
  if (init_str == "random") {
    init_method = Kmeans::InitMethod::random;
  } else if (init_str == "plusplus") {
    init_method = Kmeans::InitMethod::plus_plus;
  } else {
    std::printf("Invalid init method: %s\n", init_str.c_str());
    return 1;
  }
  Kmeans::Kernel kernel;
  if (kernel_str == "linear") {
    kernel = Kmeans::Kernel::linear;
  } else if (kernel_str == "polynomial") {
    kernel = Kmeans::Kernel::polynomial;
  } else if (kernel_str == "sigmoid") {
    kernel = Kmeans::Kernel::sigmoid;
  } else if (kernel_str == "gaussian") {
    kernel = Kmeans::Kernel::gaussian;
  } else {
    std::printf("Invalid kernel: %s\n", kernel_str.c_str());
    return 1;
  }
  Kmeans::KernelParams kp;
  kp.sigma = get_float(args, "sigma", 1.0f);
  const bool profile = args.count("profile") != 0;

  double tot_time = 0, init_time = 0, score = 0;
  try {
    for (uint32_t i = 0; i < runs; ++i) {
      const auto init_start = std::chrono::high_resolution_clock::now();
      Kmeans kmeans(n, d, k, tol, &seed, input->data(), input->clusters(), init_method, kernel, level,
                    precision, kp);
      const auto init_end = std::chrono::high_resolution_clock::now();
      if (i > 0) init_time += std::chrono::duration<double>(init_end - init_start).count();

      const auto start = std::chrono::high_resolution_clock::now();
      const uint64_t converged = kmeans.run(maxiter, check_converged);
      const auto end = std::chrono::high_resolution_clock::now();
      const double secs = std::chrono::duration<double>(end - start).count();
      if (i > 0) tot_time += secs;

      if (profile && kernel == Kmeans::Kernel::linear) {
        // distance GEMM + fused argmin + refinement; the argmin has no
        // separate kernel; label sort + centroid sums + finalize
        const std::vector<double> ms = kmeans.profile_stages(3);
        std::printf("%s[PERFORMANCE]%s compute_distances time: %.8f\n", CYAN, RESET, (ms[0] + ms[1]) / 1000);
        std::printf("%s[PERFORMANCE]%s clusters_argmin_shfl time: %.8f\n", CYAN, RESET, 0.0);
        std::printf("%s[PERFORMANCE]%s compute_centroids time: %.8f\n", CYAN, RESET,
                    (ms[2] + ms[3] + ms[4]) / 1000);
      }
      uint64_t free_b = 0, total_b = 0;
      if (km_mem_info(0, &free_b, &total_b) == KM_OK)
        std::printf("MEMORY FOOTPRINT: %llu MB\n", static_cast<unsigned long long>((total_b - free_b) / 1000000));
      if (converged < maxiter)
        std::printf("K-means converged at iteration %lu - ", static_cast<unsigned long>(converged));
      else
        std::printf("K-means did NOT converge - ");
      std::printf("Time: %lf\n", secs);
      std::printf("Objective score: %lf\n", static_cast<double>(kmeans.get_score()));
      score += kmeans.get_score();
    }
  } catch (const KmeansError& e) {
    std::printf("%s", RESET);
    std::fflush(stdout);
    std::cerr << e.what() << std::endl;
    return e.status == KM_ERR_NO_DEVICE ? EXIT_CUDA_DEV : EXIT_FAILURE;
  }

  std::printf("GPU_Kmeans: %lfs (%u runs)\n", tot_time / (runs - 1), runs);
  std::printf("Init_time: %lfs \n", init_time / (runs - 1));
  std::printf("Score: %lf\n", score / runs);
  std::printf("%s", RESET);
  std::fflush(stdout);

  if (out_file != "None") {
    std::ofstream fout(out_file, std::ios::out | std::ios::binary);
    input->dataset_to_csv(fout);
  }
  return 0;
}
