// Snapshot files: the state of a run and its clock, for post-processing and
// restart.
//
// The reference writes one HDF5 file per snapshot through its
// HierarchicalWriter (io/dump_snapshot_impl.hpp:21-32 -> save_full_state ->
// save_state, model/models.cpp:7-16 and model/all_variables.cpp:74-88): the
// scalar datasets "time" (double) and "n_steps" (int), one double dataset of
// length n_cells per conserved variable named "rho", "mv1", "mv2", "mv3", "E"
// (model/euler_variables.cpp:9-27), the scalar "n_avars" and one dataset
// "mq<k>" per advected variable.  Restart reads the same names back
// (io/load_snapshot.cpp:9-13, model/models.cpp:18-27).  A steady-state file
// carries the variables without "time" and "n_steps" (dump_snapshot_impl.hpp:
// 34-38).
//
// HDF5 is not available to this library, so the same datasets, under the same
// names, go into an uncompressed NumPy .npz container: a zip archive with one
// "<name>.npy" member per dataset.  numpy.load reads it directly, and h5py can
// rewrite it as HDF5 dataset for dataset.  Files are written to "<path>.tmp"
// and renamed, so a crash mid-write never leaves a truncated snapshot behind.
// The reader accepts uncompressed .npz files written by numpy.savez as well
// (including their zip64 records); compressed members are refused.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "mesh_obj.hpp"

using zfvm::fail;

namespace {

const char *const kCvarNames[5] = {"rho", "mv1", "mv2", "mv3", "E"};

// ---- CRC-32 (IEEE 802.3, reflected polynomial 0xEDB88320), as zip requires --

struct Crc32 {
  uint32_t table[256];
  Crc32() {
    for (uint32_t n = 0; n < 256; ++n) {
      uint32_t c = n;
      for (int k = 0; k < 8; ++k) c = (c & 1u) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
      table[n] = c;
    }
  }
  uint32_t update(uint32_t crc, const unsigned char *p, size_t n) const {
    uint32_t c = ~crc;
    for (size_t i = 0; i < n; ++i) c = table[(c ^ p[i]) & 0xFFu] ^ (c >> 8);
    return ~c;
  }
};

const Crc32 &crc32() {
  static const Crc32 t;
  return t;
}

// ---- little-endian byte packing (independent of the host's byte order) -----

void put16(std::vector<unsigned char> &b, uint32_t v) {
  b.push_back((unsigned char)(v & 0xFF));
  b.push_back((unsigned char)((v >> 8) & 0xFF));
}
void put32(std::vector<unsigned char> &b, uint32_t v) {
  put16(b, v & 0xFFFF);
  put16(b, v >> 16);
}
void put64(std::vector<unsigned char> &b, uint64_t v) {
  put32(b, (uint32_t)(v & 0xFFFFFFFFu));
  put32(b, (uint32_t)(v >> 32));
}
uint32_t get16(const unsigned char *p) { return (uint32_t)p[0] | ((uint32_t)p[1] << 8); }
uint32_t get32(const unsigned char *p) { return get16(p) | (get16(p + 2) << 16); }
uint64_t get64(const unsigned char *p) { return (uint64_t)get32(p) | ((uint64_t)get32(p + 4) << 32); }

// IEEE-754 binary64 values are stored little endian in .npy ('<f8').
void put_f64(std::vector<unsigned char> &b, double x) {
  uint64_t u;
  std::memcpy(&u, &x, 8);
  put64(b, u);
}
double get_f64(const unsigned char *p) {
  const uint64_t u = get64(p);
  double x;
  std::memcpy(&x, &u, 8);
  return x;
}

// ---- .npy members ------------------------------------------------------------

// Format 1.0: magic, version, header length, then a Python dict literal padded
// with spaces and a newline so the data starts on a 64-byte boundary.
std::vector<unsigned char> npy_header(const char *descr, bool scalar, uint64_t n) {
  std::string dict = std::string("{'descr': '") + descr + "', 'fortran_order': False, 'shape': (";
  if (!scalar) dict += std::to_string(n) + ",";
  dict += "), }";
  size_t total = 10 + dict.size() + 1;
  const size_t pad = (64 - total % 64) % 64;
  dict.append(pad, ' ');
  dict += '\n';
  std::vector<unsigned char> b = {0x93, 'N', 'U', 'M', 'P', 'Y', 1, 0};
  put16(b, (uint32_t)dict.size());
  b.insert(b.end(), dict.begin(), dict.end());
  return b;
}

struct Member {
  std::string name;  // without ".npy"
  std::vector<unsigned char> bytes;
};

Member npy_f64_column(const std::string &name, const double *base, int64_t n, int64_t stride) {
  Member m{name, npy_header("<f8", false, (uint64_t)n)};
  m.bytes.reserve(m.bytes.size() + (size_t)n * 8);
  for (int64_t i = 0; i < n; ++i) put_f64(m.bytes, base[i * stride]);
  return m;
}
Member npy_f64_scalar(const std::string &name, double x) {
  Member m{name, npy_header("<f8", true, 0)};
  put_f64(m.bytes, x);
  return m;
}
Member npy_i64_scalar(const std::string &name, int64_t x) {
  Member m{name, npy_header("<i8", true, 0)};
  put64(m.bytes, (uint64_t)x);
  return m;
}

// ---- zip container (stored members, no compression) --------------------------

// Time and date fields of every member: 1980-01-01 00:00, the zip epoch, so
// that equal snapshots are equal files.
constexpr uint32_t kDosTime = 0, kDosDate = (1u << 5) | 1u;

int write_zip(const std::string &path, const std::vector<Member> &members) {
  // the classic format's 32-bit sizes and offsets bound the file to 4 GiB
  uint64_t total = 22;
  for (const Member &m : members) total += 30 + 46 + 2 * (m.name.size() + 4) + m.bytes.size();
  if (total >= 0xFFFFFFFFull)
    return fail(ZFVM_EINVAL, "snapshot of " + std::to_string(total) + " bytes exceeds the 4 GiB zip limit");
  const std::string tmp = path + ".tmp";
  FILE *f = std::fopen(tmp.c_str(), "wb");
  if (!f) return fail(ZFVM_EINVAL, "cannot open " + tmp + " for writing");
  std::vector<unsigned char> central;
  uint64_t offset = 0;
  bool ok = true;
  for (const Member &m : members) {
    const std::string fname = m.name + ".npy";
    const uint32_t crc = crc32().update(0, m.bytes.data(), m.bytes.size());
    const uint32_t size = (uint32_t)m.bytes.size();
    std::vector<unsigned char> h;
    put32(h, 0x04034b50u);  // local file header
    put16(h, 20);           // version needed: 2.0
    put16(h, 0);            // flags
    put16(h, 0);            // stored
    put16(h, kDosTime);
    put16(h, kDosDate);
    put32(h, crc);
    put32(h, size);
    put32(h, size);
    put16(h, (uint32_t)fname.size());
    put16(h, 0);
    h.insert(h.end(), fname.begin(), fname.end());
    ok = ok && std::fwrite(h.data(), 1, h.size(), f) == h.size();
    ok = ok && std::fwrite(m.bytes.data(), 1, m.bytes.size(), f) == m.bytes.size();
    put32(central, 0x02014b50u);  // central directory entry
    put16(central, 20);           // made by: 2.0
    put16(central, 20);
    put16(central, 0);
    put16(central, 0);
    put16(central, kDosTime);
    put16(central, kDosDate);
    put32(central, crc);
    put32(central, size);
    put32(central, size);
    put16(central, (uint32_t)fname.size());
    put16(central, 0);  // extra
    put16(central, 0);  // comment
    put16(central, 0);  // disk
    put16(central, 0);  // internal attributes
    put32(central, 0);  // external attributes
    put32(central, (uint32_t)offset);
    central.insert(central.end(), fname.begin(), fname.end());
    offset += h.size() + m.bytes.size();
  }
  std::vector<unsigned char> end;
  put32(end, 0x06054b50u);  // end of central directory
  put16(end, 0);
  put16(end, 0);
  put16(end, (uint32_t)members.size());
  put16(end, (uint32_t)members.size());
  put32(end, (uint32_t)central.size());
  put32(end, (uint32_t)offset);
  put16(end, 0);
  ok = ok && std::fwrite(central.data(), 1, central.size(), f) == central.size();
  ok = ok && std::fwrite(end.data(), 1, end.size(), f) == end.size();
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) {
    std::remove(tmp.c_str());
    return fail(ZFVM_EINVAL, "writing " + tmp + " failed");
  }
  if (std::rename(tmp.c_str(), path.c_str()) != 0) {
    std::remove(tmp.c_str());
    return fail(ZFVM_EINVAL, "cannot rename " + tmp + " to " + path);
  }
  return ZFVM_OK;
}

// ---- reading ---------------------------------------------------------------------

struct Dataset {
  std::string descr;  // '<f8', '<i8', ...
  bool scalar = false;
  uint64_t n = 1;           // elements
  uint64_t data_off = 0;    // file offset of the first element
};

struct Archive {
  FILE *f = nullptr;
  std::string path, error;
  std::vector<std::pair<std::string, Dataset>> sets;
  ~Archive() {
    if (f) std::fclose(f);
  }
  bool read_at(uint64_t off, void *dst, size_t n) {
    if (std::fseek(f, (long)off, SEEK_SET) != 0) return false;
    return std::fread(dst, 1, n, f) == n;
  }
  const Dataset *find(const std::string &name) const {
    for (auto &kv : sets)
      if (kv.first == name) return &kv.second;
    return nullptr;
  }
};

// Value of key `key` in a .npy header dict, as its literal text.
bool dict_value(const std::string &d, const std::string &key, std::string &out) {
  const std::string k = "'" + key + "'";
  size_t p = d.find(k);
  if (p == std::string::npos) return false;
  p = d.find(':', p + k.size());
  if (p == std::string::npos) return false;
  ++p;
  while (p < d.size() && d[p] == ' ') ++p;
  if (p >= d.size()) return false;
  size_t e;
  if (d[p] == '\'') {
    e = d.find('\'', p + 1);
    if (e == std::string::npos) return false;
    out = d.substr(p + 1, e - p - 1);
  } else if (d[p] == '(') {
    e = d.find(')', p);
    if (e == std::string::npos) return false;
    out = d.substr(p + 1, e - p - 1);
  } else {
    e = d.find_first_of(",}", p);
    out = d.substr(p, e == std::string::npos ? std::string::npos : e - p);
  }
  return true;
}

bool parse_npy(Archive &A, const std::string &name, uint64_t off, uint64_t size, Dataset &ds) {
  unsigned char pre[12];
  if (size < 10 || !A.read_at(off, pre, 10) || std::memcmp(pre, "\x93NUMPY", 6) != 0) {
    A.error = name + " is not a .npy member";
    return false;
  }
  uint64_t hl, start;
  if (pre[6] == 1) {
    hl = get16(pre + 8);
    start = 10;
  } else {
    if (size < 12 || !A.read_at(off, pre, 12)) return false;
    hl = get32(pre + 8);
    start = 12;
  }
  if (start + hl > size) {
    A.error = name + ": bad .npy header";
    return false;
  }
  std::string d(hl, '\0');
  if (!A.read_at(off + start, &d[0], hl)) return false;
  std::string descr, order, shape;
  if (!dict_value(d, "descr", descr) || !dict_value(d, "fortran_order", order) || !dict_value(d, "shape", shape)) {
    A.error = name + ": bad .npy header";
    return false;
  }
  ds.descr = descr;
  ds.data_off = off + start + hl;
  ds.n = 1;
  int dims = 0;
  size_t p = 0;
  while (p < shape.size()) {
    while (p < shape.size() && (shape[p] == ' ' || shape[p] == ',')) ++p;
    if (p >= shape.size()) break;
    uint64_t v = 0;
    size_t e = p;
    for (; e < shape.size() && shape[e] >= '0' && shape[e] <= '9'; ++e) {
      if (v > (1ull << 40)) break;  // no dataset here is that long
      v = 10 * v + (uint64_t)(shape[e] - '0');
    }
    if (e == p || v > (1ull << 40) || (e < shape.size() && shape[e] != ',' && shape[e] != ' ')) {
      A.error = name + ": bad shape (" + shape + ")";
      return false;
    }
    ds.n *= v;
    if (++dims > 1) break;
    p = e;
  }
  ds.scalar = dims == 0;
  if (dims > 1 || (dims == 1 && order != "False" && ds.n > 1)) {
    A.error = name + ": only one-dimensional datasets are read";
    return false;
  }
  // item size from the type code ('<f8' -> 8); only 1, 2, 4 and 8 are types
  const char c = descr.size() == 3 ? descr[2] : '0';
  const uint64_t item = (c == '1' || c == '2' || c == '4' || c == '8') ? (uint64_t)(c - '0') : 0;
  if (item == 0 || ds.n > (size - start - hl) / item) {
    A.error = name + ": data shorter than its shape";
    return false;
  }
  return true;
}

bool open_archive(Archive &A, const std::string &path) {
  A.path = path;
  A.f = std::fopen(path.c_str(), "rb");
  if (!A.f) {
    A.error = "cannot open " + path;
    return false;
  }
  if (std::fseek(A.f, 0, SEEK_END) != 0) return false;
  const long flen = std::ftell(A.f);
  if (flen < 22) {
    A.error = path + " is not a zip archive";
    return false;
  }
  // the end-of-central-directory record sits in the last 22 + 65535 bytes
  const uint64_t tail = (uint64_t)std::min<long>(flen, 22 + 65535);
  std::vector<unsigned char> t(tail);
  if (!A.read_at((uint64_t)flen - tail, t.data(), tail)) return false;
  int64_t eocd = -1;
  for (int64_t i = (int64_t)tail - 22; i >= 0; --i)
    if (get32(&t[i]) == 0x06054b50u) {
      eocd = i;
      break;
    }
  if (eocd < 0) {
    A.error = path + " is not a zip archive";
    return false;
  }
  uint64_t n_entries = get16(&t[eocd + 10]);
  uint64_t cd_size = get32(&t[eocd + 12]);
  uint64_t cd_off = get32(&t[eocd + 16]);
  // zip64: a locator directly before the record points at the zip64 record
  if (eocd >= 20 && get32(&t[eocd - 20]) == 0x07064b50u) {
    unsigned char z[56];
    if (!A.read_at(get64(&t[eocd - 20 + 8]), z, 56) || get32(z) != 0x06064b50u) {
      A.error = path + ": bad zip64 record";
      return false;
    }
    n_entries = get64(z + 32);
    cd_size = get64(z + 40);
    cd_off = get64(z + 48);
  }
  if (cd_off > (uint64_t)flen || cd_size > (uint64_t)flen - cd_off || n_entries > cd_size / 46 + 1) {
    A.error = path + ": bad central directory";
    return false;
  }
  std::vector<unsigned char> cd(cd_size);
  if (!A.read_at(cd_off, cd.data(), cd_size)) {
    A.error = path + ": cannot read the central directory";
    return false;
  }
  size_t p = 0;
  for (uint64_t e = 0; e < n_entries; ++e) {
    if (p + 46 > cd.size() || get32(&cd[p]) != 0x02014b50u) {
      A.error = path + ": bad central directory";
      return false;
    }
    const uint32_t method = get16(&cd[p + 10]);
    uint64_t csize = get32(&cd[p + 20]), usize = get32(&cd[p + 24]);
    const uint32_t nlen = get16(&cd[p + 28]), xlen = get16(&cd[p + 30]), clen = get16(&cd[p + 32]);
    uint64_t loff = get32(&cd[p + 42]);
    if (p + 46 + nlen + xlen > cd.size()) {
      A.error = path + ": bad central directory";
      return false;
    }
    std::string fname((const char *)&cd[p + 46], nlen);
    // names from the file go into error messages: printable ASCII only
    for (char &ch : fname)
      if (ch < 0x20 || ch > 0x7e) ch = '?';
    // zip64 extra field (id 1): the 64-bit values of the saturated fields, in order
    const size_t xend = p + 46 + nlen + xlen;  // inside cd, checked above
    for (size_t q = p + 46 + nlen; q + 4 <= xend;) {
      const uint32_t id = get16(&cd[q]), len = get16(&cd[q + 2]);
      const size_t fend = std::min(q + 4 + len, xend);
      if (id == 1) {
        size_t r = q + 4;
        if (usize == 0xFFFFFFFFu && r + 8 <= fend) usize = get64(&cd[r]), r += 8;
        if (csize == 0xFFFFFFFFu && r + 8 <= fend) csize = get64(&cd[r]), r += 8;
        if (loff == 0xFFFFFFFFu && r + 8 <= fend) loff = get64(&cd[r]), r += 8;
      }
      q += 4 + len;
    }
    p += 46 + nlen + xlen + clen;
    if (fname.size() < 4 || fname.compare(fname.size() - 4, 4, ".npy") != 0) continue;
    const std::string name = fname.substr(0, fname.size() - 4);
    if (method != 0 || csize != usize) {
      A.error = path + ": member " + fname + " is compressed; write snapshots with numpy.savez, not savez_compressed";
      return false;
    }
    if (loff > (uint64_t)flen || usize > (uint64_t)flen) {
      A.error = path + ": member " + fname + " lies outside the file";
      return false;
    }
    unsigned char lh[30];
    if (!A.read_at(loff, lh, 30) || get32(lh) != 0x04034b50u) {
      A.error = path + ": bad local header of " + fname;
      return false;
    }
    const uint64_t data = loff + 30 + get16(lh + 26) + get16(lh + 28);
    Dataset ds;
    if (!parse_npy(A, name, data, usize, ds)) return false;
    A.sets.emplace_back(name, ds);
  }
  return true;
}

bool read_f64(Archive &A, const std::string &name, uint64_t n, double *dst, int64_t stride) {
  const Dataset *ds = A.find(name);
  if (!ds) {
    A.error = A.path + " has no dataset \"" + name + "\"";
    return false;
  }
  if (ds->descr != "<f8" || ds->scalar || ds->n != n) {
    A.error = A.path + ": dataset \"" + name + "\" is not " + std::to_string(n) + " little-endian doubles";
    return false;
  }
  std::vector<unsigned char> raw(n * 8);
  if (!A.read_at(ds->data_off, raw.data(), raw.size())) {
    A.error = A.path + ": cannot read \"" + name + "\"";
    return false;
  }
  for (uint64_t i = 0; i < n; ++i) dst[i * stride] = get_f64(&raw[i * 8]);
  return true;
}

// A scalar stored as an integer or float of 4 or 8 bytes, little endian.
bool read_scalar(Archive &A, const std::string &name, double *d, int64_t *i) {
  const Dataset *ds = A.find(name);
  if (!ds) {
    A.error = A.path + " has no dataset \"" + name + "\"";
    return false;
  }
  unsigned char b[8] = {0};
  const std::string &t = ds->descr;
  const bool known = t == "<f8" || t == "<i8" || t == "<u8" || t == "<i4" || t == "<u4";
  if (!known) {
    A.error = A.path + ": dataset \"" + name + "\" has unsupported type " + t;
    return false;
  }
  if (ds->n != 1 || !A.read_at(ds->data_off, b, (size_t)(t[2] - '0'))) {
    A.error = A.path + ": dataset \"" + name + "\" is not a scalar";
    return false;
  }
  if (t == "<f8") {
    const double x = get_f64(b);
    if (d) *d = x;
    if (i) *i = (int64_t)x;
  } else {
    int64_t x = t[2] == '8' ? (int64_t)get64(b) : (t[1] == 'i' ? (int64_t)(int32_t)get32(b) : (int64_t)get32(b));
    if (d) *d = (double)x;
    if (i) *i = x;
  }
  return true;
}

std::string avar_name(int k) { return "mq" + std::to_string(k); }

}  // namespace

extern "C" int zfvm_snapshot_write(const char *path, int64_t n_cells, const double *cvars, int32_t n_avars,
                                   const double *avars, int32_t with_clock, double t, int64_t n_steps) {
  if (!path || !cvars || n_cells <= 0 || n_avars < 0 || (n_avars > 0 && !avars))
    return fail(ZFVM_EINVAL, "zfvm_snapshot_write: null argument or bad size");
  try {
    std::vector<Member> m;
    if (with_clock) {
      m.push_back(npy_f64_scalar("time", t));
      m.push_back(npy_i64_scalar("n_steps", n_steps));
    }
    for (int k = 0; k < 5; ++k) m.push_back(npy_f64_column(kCvarNames[k], cvars + k, n_cells, 5));
    m.push_back(npy_i64_scalar("n_avars", n_avars));
    for (int k = 0; k < n_avars; ++k) m.push_back(npy_f64_column(avar_name(k), avars + k, n_cells, n_avars));
    return write_zip(path, m);
  } catch (const std::bad_alloc &) {
    return fail(ZFVM_ENOMEM, "zfvm_snapshot_write: host allocation failed");
  }
}

extern "C" int zfvm_snapshot_info(const char *path, int64_t *n_cells, int32_t *n_avars, int32_t *has_clock) {
  if (!path) return fail(ZFVM_EINVAL, "null argument");
  try {
  Archive A;
  if (!open_archive(A, path)) return fail(ZFVM_EINVAL, A.error.empty() ? "cannot read " + A.path : A.error);
  const Dataset *rho = A.find("rho");
  if (!rho || rho->scalar) return fail(ZFVM_EINVAL, A.path + " has no dataset \"rho\"");
  int64_t na = 0;
  if (A.find("n_avars") && !read_scalar(A, "n_avars", nullptr, &na)) return fail(ZFVM_EINVAL, A.error);
  if (na < 0 || na > (1 << 20)) return fail(ZFVM_EINVAL, A.path + ": bad n_avars");
  if (n_cells) *n_cells = (int64_t)rho->n;
  if (n_avars) *n_avars = (int32_t)na;
  if (has_clock) *has_clock = A.find("time") && A.find("n_steps");
  return ZFVM_OK;
  } catch (const std::bad_alloc &) {
    return fail(ZFVM_ENOMEM, "zfvm_snapshot_info: host allocation failed");
  } catch (const std::exception &e) {
    return fail(ZFVM_EINVAL, std::string("zfvm_snapshot_info: ") + e.what());
  }
}

extern "C" int zfvm_snapshot_read(const char *path, int64_t n_cells, double *cvars, int32_t n_avars, double *avars,
                                  double *t, int64_t *n_steps) {
  if (!path || !cvars || n_cells <= 0 || n_avars < 0 || (n_avars > 0 && !avars))
    return fail(ZFVM_EINVAL, "zfvm_snapshot_read: null argument or bad size");
  try {
    Archive A;
    if (!open_archive(A, path)) return fail(ZFVM_EINVAL, A.error.empty() ? "cannot read " + A.path : A.error);
    for (int k = 0; k < 5; ++k)
      if (!read_f64(A, kCvarNames[k], (uint64_t)n_cells, cvars + k, 5)) return fail(ZFVM_EINVAL, A.error);
    int64_t na = 0;
    if (A.find("n_avars") && !read_scalar(A, "n_avars", nullptr, &na)) return fail(ZFVM_EINVAL, A.error);
    if (na != n_avars)
      return fail(ZFVM_EINVAL, A.path + " holds " + std::to_string(na) + " advected variables, not " +
                                   std::to_string(n_avars));
    for (int k = 0; k < n_avars; ++k)
      if (!read_f64(A, avar_name(k), (uint64_t)n_cells, avars + k, n_avars)) return fail(ZFVM_EINVAL, A.error);
    if (t && !read_scalar(A, "time", t, nullptr)) return fail(ZFVM_EINVAL, A.error);
    if (n_steps && !read_scalar(A, "n_steps", nullptr, n_steps)) return fail(ZFVM_EINVAL, A.error);
    return ZFVM_OK;
  } catch (const std::bad_alloc &) {
    return fail(ZFVM_ENOMEM, "zfvm_snapshot_read: host allocation failed");
  } catch (const std::exception &e) {
    return fail(ZFVM_EINVAL, std::string("zfvm_snapshot_read: ") + e.what());
  }
}
