// io.h -- the reference's file interface: raw little-endian FP64 .dat arrays
// and the one-JSON-object-per-line out.json metadata (cuda/util.h:249-444).
#pragma once

#include <string>
#include <vector>

namespace holo_io {

struct Plane {
  double width = 1.0;
  double offset[3] = {0.0, 0.0, 0.0};
  double aspect_ratio = 1.0;
  bool randomize = false;
};

// Keys written after the reference's own on each out.json line: the pass's pair
// rate (every line) and, when the pass was checked against the FP64 sum at
// sampled targets, the relative L2 error and the largest phase error there.
struct Extra {
  double pairs_per_s = 0.0;
  bool checked = false;
  int check_targets = 0;
  double rel_l2 = 0.0, max_phase_err = 0.0;
};

// read_bytes<double> (cuda/util.h:249-283): the whole file as doubles.
// Returns false (and sets *err) if the file is missing, empty or not a
// multiple of 8 bytes.
bool read_dat(const std::string &path, std::vector<double> *out, std::string *err);
bool write_dat(const std::string &path, const double *data, size_t count, std::string *err);

// write_arrays (cuda/util.h:410-444): appends one metadata line to
// dir/out.json (the first call of the process truncates it) and writes
// dir/<k1>_amp.dat, dir/<k1>_phase.dat and dir/<k2>.dat.
bool write_arrays(const std::vector<double> &amp, const std::vector<double> &phase,
                  const std::vector<double> &pos, const std::string &k1, const std::string &k2,
                  const Plane &p, double dt, double flops, const Extra &extra,
                  const std::string &dir, std::string *err);

// The metadata line itself (write_metadata, cuda/util.h:358-396), the keys of
// `extra` appended after the reference's.
std::string metadata_line(const std::string &phasor, const std::string &pos, const Plane &p,
                          const std::vector<double> &amp, const std::vector<double> &phase,
                          double dt, double flops, long timestamp_ns,
                          const Extra &extra = Extra());

}  // namespace holo_io
