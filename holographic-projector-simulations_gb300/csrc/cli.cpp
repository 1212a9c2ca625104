// cli.cpp -- `holo`, flag- and file-compatible with the reference executable.
//
// Short options are the reference's getopt string (cuda/input.h:83) with its
// defaults (cuda/input.h:48-79); the help text follows cuda/input.h:7-39.
// File mode (-f dir) reads x0_amp.dat, x0_phase.dat, u0.dat, v0.dat and, with
// -F, w0_0.dat (falling back to the reference's w0.dat, cuda/main.cu:90) and
// writes y0_* / v0.dat and z0_0_* / w0_0.dat plus out.json into dir
// (cuda/main.cu:213-221).  Unlike the reference, -F projects z from the
// normalised projector field y at v onto w (the x -> y -> z chain); --ref-compat
// reproduces the reference's -F (z from x at u onto v, cuda/main.cu:219).
// Without -f the generated-data mode of cuda/main.cu:120-199 runs; the -Z
// projection planes of one object plane run there as one batched launch
// (holo_transform_batched) instead of one pass per plane.
//
// Long options added here: --lambda, --precision fp64|split32, --mc SUB,
// --seed S, --mc-block B, --amplitude-only (PROJECT_PHASE=0), --reference-distance,
// --ref-compat, --out DIR (generated mode, default ../tmp/ as the reference), --device,
// --shape (the generated object's shape; the reference fixes it at compile time),
// --check K (each pass compared with the FP64 kernel at K sampled targets).
// Every out.json line also carries "pairs_per_s", and with --check "check_targets",
// "rel_l2" and "max_phase_err", after the reference's keys.
//
// Exit codes: 0 success; 2 bad arguments or files; 4 non-finite output (the
// reference's check_complex exit, cuda/util.h:54-60); 3 a library error.
#include <cuda_runtime.h>
#include <getopt.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <algorithm>
#include <string>
#include <vector>

#include "gen.h"
#include "holo.h"
#include "io.h"

namespace {

constexpr int kNSqrt = 512;  // N_sqrt (cuda/macros.h:8)

template <typename T>
struct Range {
  T min, max;
};

// Shapes of the generated object (the reference's Shape, cuda/main.h:9).
enum class Shape { Line, LogLine, Circle, DottedCircle };

struct Params {
  size_t planes_obj = 1, planes_projection = 1;
  size_t n_obj = 1, n_projector = (size_t)kNSqrt * kNSqrt, n_projection = (size_t)kNSqrt * kNSqrt;
  bool n_projector_set = false;
  double aspect_projector = 1.0, aspect_projection = 1.0;
  Range<double> off_x{0.0, 0.0}, off_y{0.0, 0.0}, off_z{0.35, 0.25};
  Range<double> obj_width{1e-3, 1e-3};
  Range<double> projector_width{kNSqrt * 7e-6, kNSqrt * 7e-6};
  Range<double> projection_width{1e-3 * 1.2, 1e-3 * 1.2};
  Range<double> projection_z{0.0, 0.0};
  int algorithm = 2;
  bool quadrant = false, randomize = false;
  int streams = 8;
  std::string files;
  bool projection = false;
  // added
  double lambda = 0.65e-6;  // the reference's compile-time default LAMBDA (cuda/macros.h:23-25)
  int precision = HOLO_FP64;
  int mc_sub = 0;
  uint64_t seed = 0;
  int mc_block = 256;
  bool amplitude_only = false;
  Shape shape = Shape::Circle;  // the reference's generated object (cuda/main.cu:55)
  double reference_distance = 0.25;  // DISTANCE_REFERENCE_WAVE (cuda/macros.h:26-28)
  bool ref_compat = false;
  std::string out_dir = "../tmp/";
  int device = 0;
  int check = 0;  // targets per pass compared with the FP64 sum (0: no check)
};

void show_help(const char *p) {
  printf(
      "Usage %s [OPTION]...\n"
      "Note: for each attribute, if .max is not provided it defaults to the corresponding .min.\n"
      "\t -h       \tShow help. \n"
      "\n\tUse external data (optional)\n"
      "\t -f {dir} \t Read input files from `dir`: `x0_amp.dat, x0_phase.dat, u0.dat, v0.dat`."
      " These files should be binary arrays representing double-precision floating-point numbers.\n"
      "\t-F        \t Compute projection distribution (w0_0.dat, or w0.dat) w.r.t. the projector (v).\n"
      "\n\tPerformance parameters (accepted for compatibility; kernels are tuned automatically)\n"
      "\t-s        \tSet number of streams.\n"
      "\t-t, -T    \tSet number of source, target datapoints per thread.\n"
      "\t-b, -B    \tSet CUDA blockDim .x, .y.\n"
      "\t-g, -G    \tSet CUDA gridDim .x, .y.\n"
      "\t-p        \tSelect algorithm 1, 2 or 3 (all map to the same brute-force sum).\n"
      "\n\tGenerate data (used if `-f {dir}` is not supplied).\n"
      "\t-X, -Z    \tSet number of input, projection planes.\n"
      "\t-x, -y, -z\tSet number of input, projector, projection datapoints per plane.\n"
      "\t-a, -A    \tSet aspect ratio for projector, projection.\n"
      "\t-u, -U    \tSet .min, .max offset in x-dimension for input objects.\n"
      "\t-v, -V    \tSet .min, .max offset in y-dimension for input objects.\n"
      "\t-w, -W    \tSet .min, .max offset in z-dimension for input objects.\n"
      "\t-o, -O    \tSet .min, .max object width.\n"
      "\t-l, -L    \tSet .min, .max projector width.\n"
      "\t-n, -N    \tSet .min, .max projection width.\n"
      "\t-m, -M    \tSet .min, .max projection offset in z-dimension.\n"
      "\t-q        \tLimit projection to a single quadrant.\n"
      "\t-r        \tRandomize projector pixel positions.\n"
      "\n\tRuntime options (compile-time macros in the reference)\n"
      "\t--lambda L            \tWavelength in m (default 0.65e-6)\n"
      "\t--precision P         \tfp64 (default, the reference's arithmetic) or split32\n"
      "\t--amplitude-only      \tAmplitude-only projector with a reference wave (PROJECT_PHASE=0)\n"
      "\t--reference-distance D\tDistance of the reference wave source (default 0.25 m)\n"
      "\t--mc SUB [--seed S] [--mc-block B]\tMonte Carlo estimator: 1/SUB of the sources per block\n"
      "\t--ref-compat          \tReproduce the reference's -F (z from x at u onto v)\n"
      "\t--out DIR             \tOutput directory of the generated mode (default ../tmp/)\n"
      "\t--device D            \tCUDA device\n"
      "\t--shape S             \tGenerated object: circle (default), dotted-circle, line, log-line\n"
      "\t--check K             \tCompare each pass with the FP64 sum at K sampled targets\n"
      "\t                      \t(rel_l2 and max_phase_err in out.json)\n"
      "\n",
      p);
}

bool parse(int argc, char **argv, Params *p, int *exit_code) {
  enum { O_LAMBDA = 1000, O_PREC, O_MC, O_SEED, O_MCB, O_AMP, O_REFD, O_COMPAT, O_OUT, O_DEV,
         O_SHAPE, O_CHECK };
  static struct option longopts[] = {{"lambda", required_argument, 0, O_LAMBDA},
                                     {"precision", required_argument, 0, O_PREC},
                                     {"mc", required_argument, 0, O_MC},
                                     {"seed", required_argument, 0, O_SEED},
                                     {"mc-block", required_argument, 0, O_MCB},
                                     {"amplitude-only", no_argument, 0, O_AMP},
                                     {"reference-distance", required_argument, 0, O_REFD},
                                     {"ref-compat", no_argument, 0, O_COMPAT},
                                     {"out", required_argument, 0, O_OUT},
                                     {"device", required_argument, 0, O_DEV},
                                     {"shape", required_argument, 0, O_SHAPE},
                                     {"check", required_argument, 0, O_CHECK},
                                     {"help", no_argument, 0, 'h'},
                                     {0, 0, 0, 0}};
  int ch;
  while ((ch = getopt_long(argc, argv,
                           "X:Z:x:y:z:a:A:u:U:v:V:w:W:o:O:l:L:n:N:m:M:p:qrs:t:T:b:B:g:G:f:Fh",
                           longopts, nullptr)) != -1) {
    switch (ch) {
      case 'X': p->planes_obj = strtol(optarg, 0, 10); break;
      case 'Z': p->planes_projection = strtol(optarg, 0, 10); break;
      case 'x': p->n_obj = strtol(optarg, 0, 10); break;
      case 'y': p->n_projector = strtol(optarg, 0, 10); p->n_projector_set = true; break;
      case 'z': p->n_projection = strtol(optarg, 0, 10); break;
      case 'a': p->aspect_projector = strtod(optarg, 0); break;
      case 'A': p->aspect_projection = strtod(optarg, 0); break;
      case 'u': p->off_x.min = p->off_x.max = strtod(optarg, 0); break;
      case 'U': p->off_x.max = strtod(optarg, 0); break;
      case 'v': p->off_y.min = p->off_y.max = strtod(optarg, 0); break;
      case 'V': p->off_y.max = strtod(optarg, 0); break;
      case 'w': p->off_z.min = p->off_z.max = strtod(optarg, 0); break;
      case 'W': p->off_z.max = strtod(optarg, 0); break;
      case 'o': p->obj_width.min = p->obj_width.max = strtod(optarg, 0); break;
      case 'O': p->obj_width.max = strtod(optarg, 0); break;
      case 'l': p->projector_width.min = p->projector_width.max = strtod(optarg, 0); break;
      case 'L': p->projector_width.max = strtod(optarg, 0); break;
      case 'n': p->projection_width.min = p->projection_width.max = strtod(optarg, 0); break;
      case 'N': p->projection_width.max = strtod(optarg, 0); break;
      case 'm': p->projection_z.min = p->projection_z.max = strtod(optarg, 0); break;
      case 'M': p->projection_z.max = strtod(optarg, 0); break;
      case 'p': p->algorithm = strtol(optarg, 0, 10); break;
      case 'q': p->quadrant = true; break;
      case 'r': p->randomize = true; break;
      case 's': p->streams = strtol(optarg, 0, 10); break;
      case 't': case 'T': case 'b': case 'B': case 'g': case 'G': break;  // tuning hints
      case 'f': p->files = std::string(optarg) + "/"; break;
      case 'F': p->projection = true; break;
      case O_LAMBDA: p->lambda = strtod(optarg, 0); break;
      case O_PREC:
        if (!strcmp(optarg, "fp64")) p->precision = HOLO_FP64;
        else if (!strcmp(optarg, "split32")) p->precision = HOLO_SPLIT32;
        else { fprintf(stderr, "unknown precision %s\n", optarg); *exit_code = 2; return false; }
        break;
      case O_MC: p->mc_sub = strtol(optarg, 0, 10); break;
      case O_SEED: p->seed = strtoull(optarg, 0, 10); break;
      case O_MCB: p->mc_block = strtol(optarg, 0, 10); break;
      case O_AMP: p->amplitude_only = true; break;
      case O_REFD: p->reference_distance = strtod(optarg, 0); break;
      case O_COMPAT: p->ref_compat = true; break;
      case O_OUT: p->out_dir = std::string(optarg) + "/"; break;
      case O_DEV: p->device = strtol(optarg, 0, 10); break;
      case O_CHECK: p->check = (int)strtol(optarg, 0, 10); break;
      case O_SHAPE:
        if (!strcmp(optarg, "circle")) p->shape = Shape::Circle;
        else if (!strcmp(optarg, "dotted-circle")) p->shape = Shape::DottedCircle;
        else if (!strcmp(optarg, "line")) p->shape = Shape::Line;
        else if (!strcmp(optarg, "log-line")) p->shape = Shape::LogLine;
        else { fprintf(stderr, "unknown shape %s\n", optarg); *exit_code = 2; return false; }
        break;
      case 'h':
      default:
        show_help(argv[0]);
        *exit_code = 0;
        return false;
    }
  }
  // the reference's argument asserts (cuda/input.h:129-149), as errors
  const double nonzero = 1e-6;
  const char *bad = nullptr;
  if (!(0 < p->algorithm && p->algorithm <= 3)) bad = "-p must be 1, 2 or 3";
  else if (p->planes_obj < 1) bad = "-X must be >= 1";
  else if (p->planes_projection > 10000) bad = "-Z must be <= 10000";
  else if (p->n_projector == 0) bad = "-y must be > 0";
  else if (p->planes_projection && p->n_projection == 0) bad = "-z must be > 0";
  else if (!(p->lambda > 0.0) || !isfinite(p->lambda)) bad = "--lambda must be > 0";
  else if (p->mc_sub < 0) bad = "--mc must be >= 1";
  else if (p->check < 0) bad = "--check must be >= 0";
  else if (p->off_z.min > 0 ? !(p->off_z.min > nonzero && p->off_z.max > nonzero)
                            : !(-p->off_z.min > nonzero && -p->off_z.max > nonzero))
    bad = "object z offsets must be nonzero and of one sign";
  else if (fabs(p->off_z.min + p->projection_z.min) <= nonzero ||
           fabs(p->off_z.min + p->projection_z.max) <= nonzero ||
           fabs(p->off_z.max + p->projection_z.max) <= nonzero ||
           fabs(p->off_z.max + p->projection_z.min) <= nonzero)
    bad = "projection planes must not coincide with the projector plane";
  if (bad) {
    fprintf(stderr, "holo: %s\n", bad);
    *exit_code = 2;
    return false;
  }
  if (p->planes_projection == 0) p->n_projection = 1;
  return true;
}

double now() {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

double flops(double dt, size_t n, size_t m) { return dt > 0 ? n * m * 29.0 / dt : 0.0; }  // FLOP_PER_POINT

double lerp(Range<double> r, double ratio) { return (1 - ratio) * r.min + ratio * r.max; }

double gerp(Range<double> r, double ratio) {
  double a = r.min, b = r.max;
  if (a == b) return a;
  if (a == 0) a = 1e-12;
  if (b == 0) b = 1e-12;
  return pow(10, (1 - ratio) * log10(a) + ratio * log10(b));
}

// init::plane (cuda/init.h:89-158): lattice of cell-centred points on the device
// (gen.cu); -r adds the reference's cuRAND (XORWOW, seed 1235, 1236, ...) jitter.
bool lattice(std::vector<double> &v, const holo_io::Plane &p) {
  static unsigned int seed = 1234;
  if (p.randomize) seed++;
  return holo_gen::lattice(v.data(), v.size() / 3, p, seed) == 0;
}

// init::sparse_plane (cuda/init.h:160-234) for the reference's Shape (cuda/main.h:9),
// on the device (gen.cu): the object's points on a line, a line with geometric
// spacing, a circle, or a circle around a centre point.  Like the reference, line
// shapes set x only and the dotted circle leaves point 0 as it was (so y, and that
// point, keep the values of the previous object plane), then the x/y offset is added
// to every point.
bool object_points(std::vector<double> &u, Shape shape, double width, const double *offset,
                   double modulate) {
  static_assert((int)Shape::Line == holo_gen::kShapeLine &&
                    (int)Shape::LogLine == holo_gen::kShapeLogLine &&
                    (int)Shape::Circle == holo_gen::kShapeCircle &&
                    (int)Shape::DottedCircle == holo_gen::kShapeDottedCircle,
                "shape codes");
  return holo_gen::object_points(u.data(), u.size() / 3, (int)shape, width, offset,
                                 modulate) == 0;
}

int lib_fail(const char *what, int rc) {
  fprintf(stderr, "holo: %s failed (%d): %s\n", what, rc, holo_last_error_string());
  return 3;
}

bool finite_all(const std::vector<double> &a) {
  for (double x : a)
    if (!isfinite(x)) return false;
  return true;
}

struct Runner {
  holo_handle h;
  const Params &p;

  // --check: the FP64 sum at p.check targets spread evenly over the target list
  // against a computed pass, given as its normalised polar output (oa, op) and
  // the max |y| it was divided by (the raw field is oa * scale * e^{i op}).
  int check_field(int sign, const std::vector<double> &amp, const std::vector<double> &phase,
                  const std::vector<double> &u, const std::vector<double> &v,
                  const std::vector<double> &oa, const std::vector<double> &op, double max_abs,
                  holo_io::Extra *ex) {
    const size_t N = amp.size(), M = v.size() / 3;
    const size_t K = std::min<size_t>((size_t)p.check, M);
    if (K == 0) return 0;
    std::vector<size_t> idx(K);
    std::vector<double> vs(3 * K), y64(2 * K);
    for (size_t k = 0; k < K; ++k) {
      idx[k] = (size_t)(((double)k + 0.5) * (double)M / (double)K);
      for (int d = 0; d < 3; ++d) vs[3 * k + d] = v[3 * idx[k] + d];
    }
    const int rc = holo_transform(h, sign, p.lambda, amp.data(), phase.data(), u.data(), N,
                                  vs.data(), K, y64.data(), HOLO_FP64, nullptr);
    if (rc) return lib_fail("holo_transform (--check, FP64)", rc);
    const double scale = max_abs < 1e-6 ? 1.0 : max_abs;  // as the normalisation did
    double num = 0.0, den = 0.0, worst = 0.0;
    for (size_t k = 0; k < K; ++k) {
      const double a = oa[idx[k]] * scale, ph = op[idx[k]];
      const double re = a * cos(ph), im = a * sin(ph);
      const double dr = re - y64[2 * k], di = im - y64[2 * k + 1];
      num += dr * dr + di * di;
      den += y64[2 * k] * y64[2 * k] + y64[2 * k + 1] * y64[2 * k + 1];
      // angle of y / y64
      const double cr = re * y64[2 * k] + im * y64[2 * k + 1];
      const double ci = im * y64[2 * k] - re * y64[2 * k + 1];
      worst = std::max(worst, fabs(atan2(ci, cr)));
    }
    ex->checked = true;
    ex->check_targets = (int)K;
    ex->rel_l2 = den > 0.0 ? sqrt(num / den) : sqrt(num);
    ex->max_phase_err = worst;
    return 0;
  }

  // One timed pass: sources (amp, phase, pos) -> targets, normalised polar.  `ex`
  // receives the pair rate and, with --check, the comparison with FP64 (not for the
  // amplitude-only projector, whose output is not the transform's field).
  int pass(int sign, const std::vector<double> &amp, const std::vector<double> &phase,
           const std::vector<double> &u, const std::vector<double> &v, std::vector<double> *oa,
           std::vector<double> *op, double *dt, bool reference_wave, holo_io::Extra *ex) {
    const size_t N = amp.size(), M = v.size() / 3;
    oa->assign(M, 0.0);
    op->assign(M, 0.0);
    double max_abs = 0.0;
    const bool check = p.check > 0 && !reference_wave;
    const double t0 = now();
    int rc;
    if (sign == HOLO_BACKWARDS && p.mc_sub == 0 && !check) {
      rc = holo_project(h, p.lambda, amp.data(), phase.data(), u.data(), N, v.data(), M, nullptr,
                        0, oa->data(), op->data(), nullptr, nullptr, p.precision,
                        reference_wave ? 1 : 0, p.reference_distance, nullptr);
      if (rc) return lib_fail("holo_project", rc);
    } else {
      std::vector<double> y(2 * M);
      rc = p.mc_sub > 0
               ? holo_transform_mc(h, sign, p.lambda, amp.data(), phase.data(), u.data(), N,
                                   v.data(), M, y.data(), p.seed, p.mc_sub, p.mc_block, nullptr)
               : holo_transform(h, sign, p.lambda, amp.data(), phase.data(), u.data(), N,
                                v.data(), M, y.data(), p.precision, nullptr);
      if (rc) return lib_fail("holo_transform", rc);
      rc = holo_normalize_polar(h, y.data(), M, oa->data(), op->data(), &max_abs, nullptr);
      if (rc) return lib_fail("holo_normalize_polar", rc);
    }
    *dt = now() - t0;
    if (!finite_all(*oa) || !finite_all(*op)) {
      fprintf(stderr, "holo: non-finite output\n");
      return 4;
    }
    *ex = holo_io::Extra();
    ex->pairs_per_s = *dt > 0.0 ? (double)N * (double)M / *dt : 0.0;
    if (check) return check_field(sign, amp, phase, u, v, *oa, *op, max_abs, ex);
    return 0;
  }

  // Timed passes of independent problems (sources k -> targets k) as one batched
  // launch, each result normalised to polar; an array that several problems share
  // (the sources of a -Z stack) is uploaded once.  *dt is the time of the whole batch.
  struct Src {
    const std::vector<double> *amp, *phase, *pos;
  };
  int batch(int sign, const std::vector<Src> &src,
            const std::vector<const std::vector<double> *> &tgt,
            std::vector<std::vector<double>> *oa, std::vector<std::vector<double>> *op,
            double *dt, std::vector<holo_io::Extra> *ex) {
    const size_t P = src.size();
    std::vector<void *> bufs;
    struct Up {
      const double *host;
      size_t n;
      double *dev;
    };
    std::vector<Up> uploaded;
    bool ok = true;
    auto dev = [&](const double *hsrc, size_t n) -> double * {
      void *d = nullptr;
      if (cudaMalloc(&d, (n ? n : 1) * sizeof(double)) != cudaSuccess) {
        ok = false;
        return nullptr;
      }
      bufs.push_back(d);
      if (hsrc && n && cudaMemcpy(d, hsrc, n * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess)
        ok = false;
      return static_cast<double *>(d);
    };
    auto up = [&](const std::vector<double> &hv) -> double * {
      for (const Up &e : uploaded)
        if (e.host == hv.data() && e.n == hv.size()) return e.dev;
      double *d = dev(hv.data(), hv.size());
      uploaded.push_back({hv.data(), hv.size(), d});
      return d;
    };
    auto release = [&]() {
      for (void *d : bufs) cudaFree(d);
    };
    const double t0 = now();
    std::vector<holo_problem> probs(P);
    for (size_t k = 0; k < P && ok; ++k) {
      const size_t N = src[k].amp->size(), M = tgt[k]->size() / 3;
      double *da = up(*src[k].amp), *dp = up(*src[k].phase), *du = up(*src[k].pos);
      double *dw = up(*tgt[k]), *dz = dev(nullptr, 2 * M);
      probs[k] = holo_problem{da, dp, du, N, dw, M, sign, p.lambda, dz};
    }
    if (!ok) {
      release();
      fprintf(stderr, "holo: device buffers for the plane batch: %s\n",
              cudaGetErrorString(cudaGetLastError()));
      return 3;
    }
    int rc = holo_transform_batched(h, probs.data(), (int)P, p.precision, nullptr);
    if (rc) {
      release();
      return lib_fail("holo_transform_batched", rc);
    }
    oa->assign(P, {});
    op->assign(P, {});
    std::vector<double> max_abs(P, 0.0);
    for (size_t k = 0; k < P && rc == 0; ++k) {
      const size_t M = probs[k].M;
      std::vector<double> z(2 * M);
      if (cudaMemcpy(z.data(), probs[k].y_re_im, 2 * M * sizeof(double),
                     cudaMemcpyDeviceToHost) != cudaSuccess) {
        fprintf(stderr, "holo: copy of plane %zu failed\n", k);
        rc = 3;
        break;
      }
      (*oa)[k].assign(M, 0.0);
      (*op)[k].assign(M, 0.0);
      rc = holo_normalize_polar(h, z.data(), M, (*oa)[k].data(), (*op)[k].data(), &max_abs[k],
                                nullptr);
      if (rc) {
        rc = lib_fail("holo_normalize_polar", rc);
      } else if (!finite_all((*oa)[k]) || !finite_all((*op)[k])) {
        fprintf(stderr, "holo: non-finite output\n");
        rc = 4;
      }
    }
    *dt = now() - t0;
    release();
    // every problem is credited with the batch's pair rate (one launch ran them all)
    double pairs = 0.0;
    for (size_t k = 0; k < P; ++k) pairs += (double)probs[k].N * (double)probs[k].M;
    ex->assign(P, holo_io::Extra());
    for (size_t k = 0; k < P && rc == 0; ++k) {
      (*ex)[k].pairs_per_s = *dt > 0.0 ? pairs / *dt : 0.0;
      if (p.check > 0)
        rc = check_field(sign, *src[k].amp, *src[k].phase, *src[k].pos, *tgt[k], (*oa)[k],
                         (*op)[k], max_abs[k], &(*ex)[k]);
    }
    return rc;
  }
};

int write(const std::vector<double> &a, const std::vector<double> &ph,
          const std::vector<double> &pos, const std::string &k1, const std::string &k2,
          const holo_io::Plane &pl, double dt, double fl, const std::string &dir,
          const holo_io::Extra &ex = holo_io::Extra()) {
  std::string err;
  if (!holo_io::write_arrays(a, ph, pos, k1, k2, pl, dt, fl, ex, dir, &err)) {
    fprintf(stderr, "holo: %s\n", err.c_str());
    return 2;
  }
  return 0;
}

int file_mode(Runner &R, const Params &p) {
  std::string err;
  std::vector<double> xa, xp, u, v, w;
  const std::string d = p.files;
  if (!holo_io::read_dat(d + "x0_amp.dat", &xa, &err) ||
      !holo_io::read_dat(d + "x0_phase.dat", &xp, &err) ||
      !holo_io::read_dat(d + "u0.dat", &u, &err) || !holo_io::read_dat(d + "v0.dat", &v, &err)) {
    fprintf(stderr, "holo: %s\n", err.c_str());
    return 2;
  }
  if (xp.size() != xa.size() || u.size() != 3 * xa.size() || v.size() % 3) {
    fprintf(stderr, "holo: inconsistent input sizes (x0_amp %zu, x0_phase %zu, u0 %zu, v0 %zu)\n",
            xa.size(), xp.size(), u.size(), v.size());
    return 2;
  }
  if (p.projection && !p.ref_compat) {
    if (!holo_io::read_dat(d + "w0_0.dat", &w, &err) && !holo_io::read_dat(d + "w0.dat", &w, &err)) {
      fprintf(stderr, "holo: %s\n", err.c_str());
      return 2;
    }
  } else if (p.projection) {
    if (!holo_io::read_dat(d + "w0.dat", &w, &err) && !holo_io::read_dat(d + "w0_0.dat", &w, &err)) {
      fprintf(stderr, "holo: %s\n", err.c_str());
      return 2;
    }
  }
  if (w.size() % 3) {
    fprintf(stderr, "holo: w has %zu values, not a multiple of 3\n", w.size());
    return 2;
  }
  // M: v0.dat's point count, or -y when given (the reference pads with zeros or
  // truncates to -y, cuda/transform.cu:26-41)
  if (p.n_projector_set) v.resize(3 * p.n_projector, 0.0);
  printf("Number of input datapoints/plane: %zu\n", xa.size());
  const holo_io::Plane x_plane{1.0, {0.0, 0.0, 1.0}, 1.0, false};
  const holo_io::Plane y_plane{1.0, {0.0, 0.0, 0.0}, 1.0, false};
  const holo_io::Plane z_plane{1.0, {0.0, 0.0, 1.0}, 1.0, false};
  (void)x_plane;
  std::vector<double> ya, yp, za, zp;
  double dt = 0;
  holo_io::Extra ex;
  int rc = R.pass(HOLO_BACKWARDS, xa, xp, u, v, &ya, &yp, &dt, p.amplitude_only, &ex);
  if (rc) return rc;
  printf("y: %zu x %zu pairs in %.6f s (%.3f TFLOPS at 29 FLOP/pair)\n", xa.size(), ya.size(), dt,
         flops(dt, xa.size(), ya.size()) * 1e-12);
  if ((rc = write(ya, yp, v, "y0", "v0", y_plane, dt, flops(dt, xa.size(), ya.size()), d, ex)))
    return rc;
  if (p.projection) {
    if (p.ref_compat)
      rc = R.pass(HOLO_FORWARDS, xa, xp, u, v, &za, &zp, &dt, false, &ex);
    else
      rc = R.pass(HOLO_FORWARDS, ya, yp, v, w, &za, &zp, &dt, false, &ex);
    if (rc) return rc;
    const size_t n_src = p.ref_compat ? xa.size() : ya.size();
    printf("z: %zu x %zu pairs in %.6f s\n", n_src, za.size(), dt);
    if ((rc = write(za, zp, w, "z0_0", "w0_0", z_plane, dt, flops(dt, n_src, za.size()), d, ex)))
      return rc;
  }
  return 0;
}

int generated_mode(Runner &R, const Params &p) {
  std::vector<double> u(3 * p.n_obj), w(3 * p.n_projection);
  std::vector<double> xa(p.n_obj, 1.0), xp(p.n_obj, 0.0);
  // descending amplitudes: linspace(N, 1, 0) (cuda/main.cu:66-71, cuda/algebra.h linspace)
  if (p.n_obj > 1) {
    const double delta = (0.0 - 1.0) / (p.n_obj - 1.0);
    for (size_t i = 0; i < p.n_obj; ++i) xa[i] = 1.0 + delta * i;
  }
  // Every plane's points first, in the reference's order (object, projector lattice,
  // then its projection lattices: the -r seeds advance in that order), then the passes:
  // the object planes' x -> y passes as one batched launch, all their projection
  // planes' y -> z passes as another (cuda/main.cu:125-199 runs one pass at a time;
  // Monte Carlo and the amplitude-only projector keep one pass each), then the files
  // in the reference's order.
  struct XPlane {
    std::vector<double> u, v, ya, yp;
    holo_io::Plane x_plane, y_plane;
    std::vector<std::vector<double>> ws, zas, zps;
    std::vector<holo_io::Plane> zpl;
    double dt_y = 0.0, dt_z = 0.0;
    holo_io::Extra ex_y;
    std::vector<holo_io::Extra> ex_z;
  };
  std::vector<XPlane> X(p.planes_obj);
  for (size_t i = 0; i < p.planes_obj; ++i) {
    const double ratio = i == 0 ? 0.0 : i / ((double)p.planes_obj - 1.);
    const double obj_off[3] = {lerp(p.off_x, ratio), lerp(p.off_y, ratio), gerp(p.off_z, ratio)};
    XPlane &P = X[i];
    P.x_plane = holo_io::Plane{lerp(p.obj_width, ratio), {obj_off[0], obj_off[1], obj_off[2]},
                               1.0, false};
    // u carries over from the previous plane: line shapes set x only and the dotted
    // circle keeps point 0
    if (!object_points(u, p.shape, P.x_plane.width, obj_off, i / (double)p.planes_obj))
      return lib_fail("object points", -2);
    P.u = u;
    P.y_plane = holo_io::Plane{lerp(p.projector_width, ratio), {0, 0, 0}, p.aspect_projector,
                               p.randomize};
    P.v.assign(3 * p.n_projector, 0.0);
    if (!lattice(P.v, P.y_plane)) return lib_fail("projector lattice (CUDA / cuRAND)", -2);
    for (size_t j = 0; j < p.planes_projection; ++j) {
      const double r2 = j == 0 ? 0.0 : j / ((double)p.planes_projection - 1.);
      const double width = gerp(p.projection_width, r2), height = width / p.aspect_projection;
      const double po[3] = {p.quadrant ? width / 2. : 0., p.quadrant ? height / 2. : 0.,
                            lerp(p.projection_z, r2)};
      holo_io::Plane z_plane{width,
                             {obj_off[0] + po[0], obj_off[1] + po[1], obj_off[2] + po[2]},
                             p.aspect_projection,
                             p.randomize};
      if (!lattice(w, z_plane)) return lib_fail("projection lattice (CUDA / cuRAND)", -2);
      P.ws.push_back(w);
      P.zpl.push_back(z_plane);
    }
  }
  int rc;
  // x -> y
  if (X.size() > 1 && p.mc_sub == 0 && !p.amplitude_only) {
    std::vector<Runner::Src> src;
    std::vector<const std::vector<double> *> tgt;
    for (XPlane &P : X) {
      src.push_back({&xa, &xp, &P.u});
      tgt.push_back(&P.v);
    }
    std::vector<std::vector<double>> yas, yps;
    std::vector<holo_io::Extra> exs;
    double dt = 0.0;
    if ((rc = R.batch(HOLO_BACKWARDS, src, tgt, &yas, &yps, &dt, &exs))) return rc;
    for (size_t i = 0; i < X.size(); ++i) {
      X[i].ya.swap(yas[i]);
      X[i].yp.swap(yps[i]);
      X[i].dt_y = dt / (double)X.size();
      X[i].ex_y = exs[i];
    }
  } else {
    for (XPlane &P : X)
      if ((rc = R.pass(HOLO_BACKWARDS, xa, xp, P.u, P.v, &P.ya, &P.yp, &P.dt_y,
                       p.amplitude_only, &P.ex_y)))
        return rc;
  }
  // y -> z, every projection plane of every object plane
  size_t n_z = 0;
  for (const XPlane &P : X) n_z += P.ws.size();
  if (n_z > 1 && p.mc_sub == 0) {
    std::vector<Runner::Src> src;
    std::vector<const std::vector<double> *> tgt;
    for (XPlane &P : X)
      for (const std::vector<double> &wj : P.ws) {
        src.push_back({&P.ya, &P.yp, &P.v});
        tgt.push_back(&wj);
      }
    std::vector<std::vector<double>> zas, zps;
    std::vector<holo_io::Extra> exs;
    double dt = 0.0;
    if ((rc = R.batch(HOLO_FORWARDS, src, tgt, &zas, &zps, &dt, &exs))) return rc;
    size_t k = 0;
    for (XPlane &P : X) {
      P.dt_z = dt / (double)n_z;
      for (size_t j = 0; j < P.ws.size(); ++j, ++k) {
        P.zas.push_back(std::move(zas[k]));
        P.zps.push_back(std::move(zps[k]));
        P.ex_z.push_back(exs[k]);
      }
    }
  } else {
    for (XPlane &P : X)
      for (const std::vector<double> &wj : P.ws) {
        std::vector<double> za, zp;
        holo_io::Extra ex;
        if ((rc = R.pass(HOLO_FORWARDS, P.ya, P.yp, P.v, wj, &za, &zp, &P.dt_z, false, &ex)))
          return rc;
        P.zas.push_back(std::move(za));
        P.zps.push_back(std::move(zp));
        P.ex_z.push_back(ex);
      }
  }
  for (size_t i = 0; i < X.size(); ++i) {
    const XPlane &P = X[i];
    const std::string xs = std::to_string(i);
    if ((rc = write(xa, xp, P.u, "x" + xs, "u" + xs, P.x_plane, 0.0, 0.0, p.out_dir))) return rc;
    if ((rc = write(P.ya, P.yp, P.v, "y" + xs, "v" + xs, P.y_plane, P.dt_y,
                    flops(P.dt_y, xa.size(), P.ya.size()), p.out_dir, P.ex_y)))
      return rc;
    for (size_t j = 0; j < P.ws.size(); ++j) {
      const std::string zs = xs + "_" + std::to_string(j);
      if ((rc = write(P.zas[j], P.zps[j], P.ws[j], "z" + zs, "w" + zs, P.zpl[j], P.dt_z,
                      flops(P.dt_z, P.ya.size(), P.zas[j].size()), p.out_dir, P.ex_z[j])))
        return rc;
    }
  }
  return 0;
}

}  // namespace

int main(int argc, char **argv) {
  Params p;
  int code = 0;
  if (!parse(argc, argv, &p, &code)) return code;
  holo_handle h = nullptr;
  int rc = holo_create(p.device, &h);
  if (rc) return lib_fail("holo_create", rc);
  Runner R{h, p};
  rc = p.files.empty() ? generated_mode(R, p) : file_mode(R, p);
  holo_destroy(h);
  if (rc == 0) printf("done\n");
  return rc;
}
