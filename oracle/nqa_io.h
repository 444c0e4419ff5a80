/* Named-array container used by the oracle tools and the golden fixtures.
 *
 * Layout: "NQA1", then records of
 *   u32 name_len | name bytes | u8 dtype (0=i32 1=f64 2=i64 3=f32 4=u8) | u64 count | payload
 * all little-endian.  The Python side is tests/nqa.py.  Test infrastructure only. */
#ifndef NQ_ORACLE_NQA_IO_H
#define NQ_ORACLE_NQA_IO_H
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

namespace nqa {
struct Array {
  uint8_t dtype = 1;
  std::vector<uint8_t> bytes;
  size_t count() const {
    static const size_t sz[5] = {4, 8, 8, 4, 1};
    return bytes.size() / sz[dtype];
  }
  template <class T> std::vector<T> as() const;
};

template <class T> static inline uint8_t code();
template <> inline uint8_t code<int32_t>() { return 0; }
template <> inline uint8_t code<double>() { return 1; }
template <> inline uint8_t code<int64_t>() { return 2; }
template <> inline uint8_t code<float>() { return 3; }
template <> inline uint8_t code<uint8_t>() { return 4; }

template <class S, class T> static void conv(const uint8_t *p, size_t n, std::vector<T> &out) {
  out.resize(n);
  for (size_t i = 0; i < n; ++i) {
    S v;
    std::memcpy(&v, p + i * sizeof(S), sizeof(S));
    out[i] = (T)v;
  }
}

template <class T> std::vector<T> Array::as() const {
  std::vector<T> out;
  size_t n = count();
  switch (dtype) {
  case 0: conv<int32_t>(bytes.data(), n, out); break;
  case 1: conv<double>(bytes.data(), n, out); break;
  case 2: conv<int64_t>(bytes.data(), n, out); break;
  case 3: conv<float>(bytes.data(), n, out); break;
  default: conv<uint8_t>(bytes.data(), n, out); break;
  }
  return out;
}

struct File {
  std::map<std::string, Array> arrays;
  std::vector<std::string> order;

  bool has(const std::string &k) const { return arrays.count(k) > 0; }
  const Array &get(const std::string &k) const {
    auto it = arrays.find(k);
    if (it == arrays.end()) throw std::runtime_error("nqa: missing array " + k);
    return it->second;
  }
  template <class T> std::vector<T> vec(const std::string &k) const { return get(k).as<T>(); }
  double scalar(const std::string &k, double dflt) const { return has(k) ? vec<double>(k).at(0) : dflt; }

  template <class T> void put(const std::string &k, const T *p, size_t n) {
    Array a;
    a.dtype = code<T>();
    a.bytes.resize(n * sizeof(T));
    if (n) std::memcpy(a.bytes.data(), p, n * sizeof(T));
    if (!arrays.count(k)) order.push_back(k);
    arrays[k] = a;
  }
  template <class T> void put(const std::string &k, const std::vector<T> &v) { put(k, v.data(), v.size()); }
  void put_scalar(const std::string &k, double v) { put(k, &v, 1); }

  void load(const std::string &path) {
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) throw std::runtime_error("nqa: cannot open " + path);
    char magic[4];
    if (std::fread(magic, 1, 4, f) != 4 || std::memcmp(magic, "NQA1", 4) != 0) {
      std::fclose(f);
      throw std::runtime_error("nqa: bad magic in " + path);
    }
    for (;;) {
      uint32_t nl;
      if (std::fread(&nl, 4, 1, f) != 1) break;
      std::string name(nl, '\0');
      uint8_t dt;
      uint64_t cnt;
      if (std::fread(&name[0], 1, nl, f) != nl || std::fread(&dt, 1, 1, f) != 1 || std::fread(&cnt, 8, 1, f) != 1) {
        std::fclose(f);
        throw std::runtime_error("nqa: truncated " + path);
      }
      static const size_t sz[5] = {4, 8, 8, 4, 1};
      Array a;
      a.dtype = dt;
      a.bytes.resize(cnt * sz[dt]);
      if (cnt && std::fread(a.bytes.data(), 1, a.bytes.size(), f) != a.bytes.size()) {
        std::fclose(f);
        throw std::runtime_error("nqa: truncated payload " + path);
      }
      if (!arrays.count(name)) order.push_back(name);
      arrays[name] = a;
    }
    std::fclose(f);
  }

  void save(const std::string &path) const {
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) throw std::runtime_error("nqa: cannot write " + path);
    std::fwrite("NQA1", 1, 4, f);
    static const size_t sz[5] = {4, 8, 8, 4, 1};
    for (const auto &k : order) {
      const Array &a = arrays.at(k);
      uint32_t nl = (uint32_t)k.size();
      uint64_t cnt = a.bytes.size() / sz[a.dtype];
      std::fwrite(&nl, 4, 1, f);
      std::fwrite(k.data(), 1, nl, f);
      std::fwrite(&a.dtype, 1, 1, f);
      std::fwrite(&cnt, 8, 1, f);
      if (!a.bytes.empty()) std::fwrite(a.bytes.data(), 1, a.bytes.size(), f);
    }
    std::fclose(f);
  }
};
} // namespace nqa
#endif
