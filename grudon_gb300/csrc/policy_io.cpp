// Round-policy model files for C/C++ hosts: the JSON layout the Python
// package writes ({"model": {"mean": [...], "scale": [...], "w1": [...], ...},
// "meta": {...}}), read and written field by field.  Weights are fp16 bit
// patterns (integers), the rest floats.
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/grudon_gpu.h"

namespace {

bool read_file(const char* path, std::string& out) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  char buf[1 << 16];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) out.append(buf, n);
  const bool ok = !std::ferror(f);
  std::fclose(f);
  return ok;
}

// Parses the number list of "name": [ ... ] inside the "model" object.
template <class T>
bool parse_field(const std::string& s, size_t model_at, const char* name, T* dst, size_t count) {
  const std::string key = std::string("\"") + name + "\"";
  const size_t k = s.find(key, model_at);
  if (k == std::string::npos) return false;
  size_t p = s.find('[', k + key.size());
  if (p == std::string::npos) return false;
  ++p;
  for (size_t i = 0; i < count; ++i) {
    while (p < s.size() && (s[p] == ' ' || s[p] == ',' || s[p] == '\n' || s[p] == '\r' || s[p] == '\t')) ++p;
    if (p >= s.size() || s[p] == ']') return false;
    const char* b = s.c_str() + p;
    char* e = nullptr;
    errno = 0;
    const double v = std::strtod(b, &e);
    if (e == b || errno == ERANGE) return false;
    dst[i] = (T)v;
    p += (size_t)(e - b);
  }
  while (p < s.size() && (s[p] == ' ' || s[p] == '\n' || s[p] == '\r' || s[p] == '\t')) ++p;
  return p < s.size() && s[p] == ']';
}

template <class T>
void write_field(FILE* f, const char* name, const T* v, size_t count, bool integer, bool last) {
  std::fprintf(f, "\"%s\": [", name);
  for (size_t i = 0; i < count; ++i) {
    if (integer)
      std::fprintf(f, "%s%u", i ? ", " : "", (unsigned)v[i]);
    else
      std::fprintf(f, "%s%.9g", i ? ", " : "", (double)v[i]);
  }
  std::fprintf(f, "]%s", last ? "" : ", ");
}

}  // namespace

extern "C" {

int grd_policy_load(const char* path, grd_policy_model* out) {
  if (!path || !out) return GRD_E_INVALID;
  std::string s;
  if (!read_file(path, s)) return GRD_E_IO;
  const size_t m = s.find("\"model\"");
  if (m == std::string::npos) return GRD_E_IO;
  grd_policy_model t{};
  const bool ok = parse_field(s, m, "mean", t.mean, GRD_POLICY_IN) &&
                  parse_field(s, m, "scale", t.scale, GRD_POLICY_IN) &&
                  parse_field(s, m, "w1", t.w1, GRD_POLICY_HID * GRD_POLICY_IN) &&
                  parse_field(s, m, "b1", t.b1, GRD_POLICY_HID) &&
                  parse_field(s, m, "w2", t.w2, GRD_POLICY_HID * GRD_POLICY_HID) &&
                  parse_field(s, m, "b2", t.b2, GRD_POLICY_HID) &&
                  parse_field(s, m, "w3", t.w3, GRD_POLICY_OUT * GRD_POLICY_HID) &&
                  parse_field(s, m, "b3", t.b3, GRD_POLICY_OUT);
  if (!ok) return GRD_E_IO;
  // files without a training range: no clamping
  if (s.find("\"lo\"", m) == std::string::npos && s.find("\"hi\"", m) == std::string::npos) {
    for (int i = 0; i < GRD_POLICY_IN; ++i) t.lo[i] = -1e30f, t.hi[i] = 1e30f;
  } else if (!parse_field(s, m, "lo", t.lo, GRD_POLICY_IN) || !parse_field(s, m, "hi", t.hi, GRD_POLICY_IN)) {
    return GRD_E_IO;
  }
  *out = t;
  return GRD_OK;
}

int grd_policy_save(const char* path, const grd_policy_model* m) {
  if (!path || !m) return GRD_E_INVALID;
  FILE* f = std::fopen(path, "w");
  if (!f) return GRD_E_IO;
  std::fprintf(f, "{\"model\": {");
  write_field(f, "mean", m->mean, GRD_POLICY_IN, false, false);
  write_field(f, "scale", m->scale, GRD_POLICY_IN, false, false);
  write_field(f, "w1", m->w1, GRD_POLICY_HID * GRD_POLICY_IN, true, false);
  write_field(f, "b1", m->b1, GRD_POLICY_HID, false, false);
  write_field(f, "w2", m->w2, GRD_POLICY_HID * GRD_POLICY_HID, true, false);
  write_field(f, "b2", m->b2, GRD_POLICY_HID, false, false);
  write_field(f, "w3", m->w3, GRD_POLICY_OUT * GRD_POLICY_HID, true, false);
  write_field(f, "b3", m->b3, GRD_POLICY_OUT, false, false);
  write_field(f, "lo", m->lo, GRD_POLICY_IN, false, false);
  write_field(f, "hi", m->hi, GRD_POLICY_IN, false, true);
  std::fprintf(f, "}, \"meta\": {}}\n");
  const bool ok = std::fclose(f) == 0;
  return ok ? GRD_OK : GRD_E_IO;
}

}  // extern "C"
