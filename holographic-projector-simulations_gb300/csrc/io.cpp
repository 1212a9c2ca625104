// io.cpp -- .dat and out.json, byte-compatible with the reference
// (cuda/util.h:249-283 read_bytes, :296-337 writers, :358-396 write_metadata,
// :410-444 write_arrays).  Arrays are written with one fwrite instead of the
// reference's per-byte ostream_iterator copies.
#include "io.h"

#include <math.h>
#include <stdio.h>
#include <time.h>

#include <sstream>

namespace holo_io {

bool read_dat(const std::string &path, std::vector<double> *out, std::string *err) {
  FILE *f = fopen(path.c_str(), "rb");
  if (!f) {
    *err = "cannot open " + path;
    return false;
  }
  fseek(f, 0, SEEK_END);
  const long size = ftell(f);
  fseek(f, 0, SEEK_SET);
  if (size <= 0 || size % (long)sizeof(double) != 0) {
    fclose(f);
    *err = path + ": size " + std::to_string(size) + " is not a positive multiple of 8 bytes";
    return false;
  }
  out->resize((size_t)size / sizeof(double));
  const size_t got = fread(out->data(), sizeof(double), out->size(), f);
  fclose(f);
  if (got != out->size()) {
    *err = "short read on " + path;
    return false;
  }
  return true;
}

bool write_dat(const std::string &path, const double *data, size_t count, std::string *err) {
  FILE *f = fopen(path.c_str(), "wb");
  if (!f) {
    *err = "cannot write " + path;
    return false;
  }
  const size_t put = count ? fwrite(data, sizeof(double), count, f) : 0;
  fclose(f);
  if (put != count) {
    *err = "short write on " + path;
    return false;
  }
  return true;
}

std::string metadata_line(const std::string &phasor, const std::string &pos, const Plane &p,
                          const std::vector<double> &amp, const std::vector<double> &phase,
                          double dt, double flops, long timestamp_ns, const Extra &extra) {
  // sums in array order (transform_reduce, cuda/algebra.h), default ostream
  // formatting as in the reference (its std::fixed is set after this line)
  double a = 0.0, ph = 0.0;
  for (double v : amp) a += v;
  for (double v : phase) ph += v;
  std::ostringstream out;
  const char *s1 = ": ", *s2 = ", ";
  out << "{"
      << "\"phasor\"" << s1 << "\"" << phasor << "\"" << s2
      << "\"amp_sum\"" << s1 << a << s2
      << "\"phase_sum\"" << s1 << ph << s2
      << "\"pos\"" << s1 << "\"" << pos << "\"" << s2
      << "\"len\"" << s1 << amp.size() << s2
      << "\"precision\"" << s1 << 8 << s2
      << "\"dims\"" << s1 << 3 << s2
      << "\"x_offset\"" << s1 << p.offset[0] << s2
      << "\"y_offset\"" << s1 << p.offset[1] << s2
      << "\"z_offset\"" << s1 << p.offset[2] << s2
      << "\"width\"" << s1 << p.width << s2
      << "\"randomized\"" << s1 << (p.randomize ? 1 : 0) << s2
      << "\"aspect_ratio\"" << s1 << p.aspect_ratio << s2
      << "\"timestamp\"" << s1 << timestamp_ns << s2
      << "\"runtime\"" << s1 << dt << s2
      << "\"flops\"" << s1 << flops << s2
      << "\"pairs_per_s\"" << s1 << extra.pairs_per_s;
  if (extra.checked)
    out << s2 << "\"check_targets\"" << s1 << extra.check_targets << s2
        << "\"rel_l2\"" << s1 << extra.rel_l2 << s2
        << "\"max_phase_err\"" << s1 << extra.max_phase_err;
  out << "}\n";
  return out.str();
}

bool write_arrays(const std::vector<double> &amp, const std::vector<double> &phase,
                  const std::vector<double> &pos, const std::string &k1, const std::string &k2,
                  const Plane &p, double dt, double flops, const Extra &extra,
                  const std::string &dir, std::string *err) {
  static bool overwrite = true;  // the first call of the process truncates out.json
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  const std::string line = metadata_line(k1, k2, p, amp, phase, dt, flops, (long)t.tv_nsec, extra);
  FILE *f = fopen((dir + "out.json").c_str(), overwrite ? "wb" : "ab");
  if (!f) {
    *err = "cannot write " + dir + "out.json";
    return false;
  }
  fwrite(line.data(), 1, line.size(), f);
  fclose(f);
  overwrite = false;
  if (!write_dat(dir + k1 + "_amp.dat", amp.data(), amp.size(), err)) return false;
  if (!write_dat(dir + k1 + "_phase.dat", phase.data(), phase.size(), err)) return false;
  if (!write_dat(dir + k2 + ".dat", pos.data(), pos.size(), err)) return false;
  return true;
}

}  // namespace holo_io
