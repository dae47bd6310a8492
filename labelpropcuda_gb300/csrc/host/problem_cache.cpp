// Binary cache of generated problems. Generating the 20 M-vertex input takes
// tens of seconds (the reference's generator writes its graph as text and
// never reads it back, src/generateSparseGraph.cu:218-274); a cache file
// holds one problem exactly as generated, keyed by the generator arguments,
// and is read back in the time it takes to read its bytes.
//
// File layout (little-endian, as on every target here; a byte-order word is
// checked on load):
//   header   CacheHeader below
//   payload  row_ptr[n + 1] i32, col[m] i32, val[m] f32, truth[n] f32, then
//            per batch: four i32 counts (inserted, gt, deleted, edges) and
//            inserted i32, gt_ids i32, gt_labels f32, deleted i32,
//            edge_src i32, edge_dst i32, edge_w f32
// The header carries the payload size and a 64-bit hash of the payload; a
// file whose key, size or hash does not match is not used.
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <unistd.h>

#include "problem.h"

namespace dlp {

namespace {

constexpr char kMagic[8] = {'D', 'L', 'P', 'P', 'R', 'O', 'B', '1'};
constexpr uint32_t kFormat = 1;
constexpr uint32_t kByteOrder = 0x01020304u;

struct CacheHeader {
  char magic[8];
  uint32_t format;
  uint32_t byte_order;
  ProblemKey key;
  int64_t num_edges;
  uint64_t payload_bytes;
  uint64_t hash;
};

// Word-wise multiply-xor hash (the 64-bit finaliser of MurmurHash3 applied
// per 8-byte word); detects truncation and corruption, not tampering.
struct Hasher {
  uint64_t h = 0x9e3779b97f4a7c15ull;
  void add(const void *data, size_t bytes) {
    const unsigned char *p = static_cast<const unsigned char *>(data);
    size_t i = 0;
    for (; i + 8 <= bytes; i += 8) {
      uint64_t w;
      std::memcpy(&w, p + i, 8);
      mix(w);
    }
    if (i < bytes) {
      uint64_t w = 0;
      std::memcpy(&w, p + i, bytes - i);
      mix(w ^ (static_cast<uint64_t>(bytes - i) << 56));
    }
  }
  void mix(uint64_t w) {
    w ^= w >> 33;
    w *= 0xff51afd7ed558ccdull;
    w ^= w >> 33;
    h = (h ^ w) * 0xc4ceb9fe1a85ec53ull;
    h ^= h >> 29;
  }
};

bool same_key(const ProblemKey &a, const ProblemKey &b) { return std::memcmp(&a, &b, sizeof(ProblemKey)) == 0; }

class Writer {
 public:
  explicit Writer(FILE *f) : f_(f) {}
  template <class T>
  void put(const std::vector<T> &v) { put_raw(v.data(), v.size() * sizeof(T)); }
  void put_i32(int32_t x) { put_raw(&x, sizeof(x)); }
  void put_raw(const void *p, size_t bytes) {
    if (!ok_ || bytes == 0) return;
    hash_.add(p, bytes);
    ok_ = std::fwrite(p, 1, bytes, f_) == bytes;
    bytes_ += bytes;
  }
  bool ok() const { return ok_; }
  uint64_t bytes() const { return bytes_; }
  uint64_t hash() const { return hash_.h; }

 private:
  FILE *f_;
  Hasher hash_;
  bool ok_ = true;
  uint64_t bytes_ = 0;
};

class Reader {
 public:
  Reader(FILE *f, uint64_t payload) : f_(f), left_(payload) {}
  template <class T>
  bool get(std::vector<T> &v, int64_t count) {
    if (count < 0 || static_cast<uint64_t>(count) > left_ / sizeof(T)) return ok_ = false;
    v.resize(static_cast<size_t>(count));
    return get_raw(v.data(), v.size() * sizeof(T));
  }
  bool get_i32(int32_t &x) { return get_raw(&x, sizeof(x)); }
  bool get_raw(void *p, size_t bytes) {
    if (!ok_ || bytes > left_) return ok_ = false;
    if (bytes == 0) return true;
    ok_ = std::fread(p, 1, bytes, f_) == bytes;
    if (ok_) hash_.add(p, bytes);
    left_ -= bytes;
    return ok_;
  }
  bool done() const { return ok_ && left_ == 0; }
  uint64_t hash() const { return hash_.h; }

 private:
  FILE *f_;
  Hasher hash_;
  bool ok_ = true;
  uint64_t left_;
};

bool set(std::string *err, const std::string &msg) {
  if (err) *err = msg;
  return false;
}

}  // namespace

std::string cache_file_name(const ProblemKey &k) {
  char buf[160];
  std::snprintf(buf, sizeof(buf), "dlp_problem_n%d_d%d_b%d_s%u_gt%08x_del%08x_g%u.bin", k.num_nodes, k.avg_degree,
                k.num_batches, k.seed, k.gt_fraction_bits, k.deleted_fraction_bits, k.generator);
  return buf;
}

bool save_problem(const Problem &p, const ProblemKey &key, const std::string &path, std::string *err) {
  // written under a temporary name, then renamed: a reader never sees a
  // partial file, and two writers of the same key leave one whole file
  const std::string tmp = path + ".tmp." + std::to_string(static_cast<long>(getpid()));
  FILE *f = std::fopen(tmp.c_str(), "wb");
  if (!f) return set(err, "cannot create " + tmp + ": " + std::strerror(errno));
  CacheHeader h{};
  std::memcpy(h.magic, kMagic, sizeof(kMagic));
  h.format = kFormat;
  h.byte_order = kByteOrder;
  h.key = key;
  h.num_edges = p.graph.num_edges();
  bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1;  // rewritten with the size and hash below
  Writer w(f);
  w.put(p.graph.row_ptr);
  w.put(p.graph.col);
  w.put(p.graph.val);
  w.put(p.truth);
  for (const HostBatch &b : p.batches) {
    w.put_i32(static_cast<int32_t>(b.inserted.size()));
    w.put_i32(static_cast<int32_t>(b.gt_ids.size()));
    w.put_i32(static_cast<int32_t>(b.deleted.size()));
    w.put_i32(static_cast<int32_t>(b.edge_src.size()));
    w.put(b.inserted);
    w.put(b.gt_ids);
    w.put(b.gt_labels);
    w.put(b.deleted);
    w.put(b.edge_src);
    w.put(b.edge_dst);
    w.put(b.edge_w);
  }
  h.payload_bytes = w.bytes();
  h.hash = w.hash();
  ok = ok && w.ok() && std::fseek(f, 0, SEEK_SET) == 0 && std::fwrite(&h, sizeof(h), 1, f) == 1;
  ok = (std::fclose(f) == 0) && ok;
  if (!ok || std::rename(tmp.c_str(), path.c_str()) != 0) {
    std::remove(tmp.c_str());
    return set(err, "cannot write " + path);
  }
  return true;
}

bool load_problem(const std::string &path, const ProblemKey *want, Problem &p, ProblemKey *key_out,
                  std::string *err) {
  FILE *f = std::fopen(path.c_str(), "rb");
  if (!f) return set(err, "cannot open " + path + ": " + std::strerror(errno));
  CacheHeader h{};
  bool ok = std::fread(&h, sizeof(h), 1, f) == 1;
  std::string why;
  if (!ok) why = "short header";
  else if (std::memcmp(h.magic, kMagic, sizeof(kMagic)) != 0) why = "not a problem cache file";
  else if (h.format != kFormat) why = "unknown format " + std::to_string(h.format);
  else if (h.byte_order != kByteOrder) why = "byte order differs";
  else if (want && !same_key(h.key, *want)) why = "generator arguments differ";
  else if (h.key.num_nodes < 0 || h.key.num_batches < 0 || h.num_edges < 0) why = "invalid sizes";
  if (why.empty()) {
    // the payload must be exactly the rest of the file
    const long at = std::ftell(f);
    if (std::fseek(f, 0, SEEK_END) != 0) why = "cannot seek";
    else if (static_cast<uint64_t>(std::ftell(f) - at) != h.payload_bytes) why = "size differs from its header";
    else if (std::fseek(f, at, SEEK_SET) != 0) why = "cannot seek";
  }
  if (!why.empty()) {
    std::fclose(f);
    return set(err, path + ": " + why);
  }
  Problem q;
  Reader r(f, h.payload_bytes);
  const int n = h.key.num_nodes;
  q.graph.n = n;
  ok = r.get(q.graph.row_ptr, static_cast<int64_t>(n) + 1) && r.get(q.graph.col, h.num_edges) &&
       r.get(q.graph.val, h.num_edges) && r.get(q.truth, n);
  q.batches.resize(static_cast<size_t>(h.key.num_batches));
  for (HostBatch &b : q.batches) {
    if (!ok) break;
    int32_t ni = 0, ng = 0, nd = 0, ne = 0;
    ok = r.get_i32(ni) && r.get_i32(ng) && r.get_i32(nd) && r.get_i32(ne) && r.get(b.inserted, ni) &&
         r.get(b.gt_ids, ng) && r.get(b.gt_labels, ng) && r.get(b.deleted, nd) && r.get(b.edge_src, ne) &&
         r.get(b.edge_dst, ne) && r.get(b.edge_w, ne);
  }
  std::fclose(f);
  if (!ok || !r.done()) return set(err, path + ": truncated or inconsistent payload");
  if (r.hash() != h.hash) return set(err, path + ": payload hash differs from its header");
  // the CSR must be usable as is: monotone row pointers ending at the edge count
  if (q.graph.row_ptr[0] != 0 || q.graph.row_ptr[n] != h.num_edges)
    return set(err, path + ": row pointers do not match the edge count");
  for (int i = 0; i < n; ++i)
    if (q.graph.row_ptr[i] > q.graph.row_ptr[i + 1]) return set(err, path + ": row pointers not monotone");
  p = std::move(q);
  if (key_out) *key_out = h.key;
  return true;
}

}  // namespace dlp
