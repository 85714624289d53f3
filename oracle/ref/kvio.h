// Named-array container ("DRKV") shared by the reference driver and the
// Python fixture tools (oracle/ref/kvio.py).  Test infrastructure only.
//
// Layout: "DRKV" magic, uint32 entry count, then per entry:
//   uint32 name length, name bytes, uint32 dtype (0 f32, 1 i32, 2 u32, 3 f64),
//   uint64 element count, raw little-endian data.
#pragma once
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

namespace kv {

enum DType : uint32_t { F32 = 0, I32 = 1, U32 = 2, F64 = 3 };

static inline size_t dtype_size(uint32_t dt) { return dt == F64 ? 8 : 4; }

struct Entry {
  uint32_t dtype = F32;
  std::vector<char> bytes;
  size_t count() const { return bytes.size() / dtype_size(dtype); }
  template <class T> const T* as() const { return reinterpret_cast<const T*>(bytes.data()); }
};

struct File {
  std::map<std::string, Entry> items;
  std::vector<std::string> order;

  bool has(const std::string& k) const { return items.count(k) != 0; }
  const Entry& get(const std::string& k) const {
    auto it = items.find(k);
    if (it == items.end()) throw std::runtime_error("missing key " + k);
    return it->second;
  }
  template <class T> std::vector<T> vec(const std::string& k) const {
    const Entry& e = get(k);
    const T* p = e.as<T>();
    return std::vector<T>(p, p + e.count());
  }
  int i(const std::string& k, int def = 0) const { return has(k) ? get(k).as<int32_t>()[0] : def; }
  float f(const std::string& k, float def = 0.f) const { return has(k) ? get(k).as<float>()[0] : def; }

  template <class T> void put(const std::string& k, uint32_t dt, const T* data, size_t n) {
    Entry e;
    e.dtype = dt;
    e.bytes.resize(n * sizeof(T));
    if (n) std::memcpy(e.bytes.data(), data, n * sizeof(T));
    if (!items.count(k)) order.push_back(k);
    items[k] = std::move(e);
  }
  void put_f32(const std::string& k, const std::vector<float>& v) { put(k, F32, v.data(), v.size()); }
  void put_i32(const std::string& k, const std::vector<int32_t>& v) { put(k, I32, v.data(), v.size()); }
  void put_u32(const std::string& k, const std::vector<uint32_t>& v) { put(k, U32, v.data(), v.size()); }
  void put_f64(const std::string& k, const std::vector<double>& v) { put(k, F64, v.data(), v.size()); }

  static File load(const char* path) {
    File f;
    FILE* fp = std::fopen(path, "rb");
    if (!fp) throw std::runtime_error(std::string("cannot open ") + path);
    char magic[4];
    uint32_t n = 0;
    if (std::fread(magic, 1, 4, fp) != 4 || std::memcmp(magic, "DRKV", 4) != 0) throw std::runtime_error("bad magic");
    if (std::fread(&n, 4, 1, fp) != 1) throw std::runtime_error("truncated");
    for (uint32_t e = 0; e < n; e++) {
      uint32_t len = 0, dt = 0;
      uint64_t cnt = 0;
      if (std::fread(&len, 4, 1, fp) != 1) throw std::runtime_error("truncated");
      std::string name(len, '\0');
      if (len && std::fread(&name[0], 1, len, fp) != len) throw std::runtime_error("truncated");
      if (std::fread(&dt, 4, 1, fp) != 1 || std::fread(&cnt, 8, 1, fp) != 1) throw std::runtime_error("truncated");
      Entry en;
      en.dtype = dt;
      en.bytes.resize(cnt * dtype_size(dt));
      if (cnt && std::fread(en.bytes.data(), 1, en.bytes.size(), fp) != en.bytes.size()) throw std::runtime_error("truncated");
      f.order.push_back(name);
      f.items[name] = std::move(en);
    }
    std::fclose(fp);
    return f;
  }

  void save(const char* path) const {
    FILE* fp = std::fopen(path, "wb");
    if (!fp) throw std::runtime_error(std::string("cannot write ") + path);
    uint32_t n = (uint32_t)order.size();
    std::fwrite("DRKV", 1, 4, fp);
    std::fwrite(&n, 4, 1, fp);
    for (const auto& k : order) {
      const Entry& e = items.at(k);
      uint32_t len = (uint32_t)k.size();
      uint64_t cnt = e.count();
      std::fwrite(&len, 4, 1, fp);
      std::fwrite(k.data(), 1, len, fp);
      std::fwrite(&e.dtype, 4, 1, fp);
      std::fwrite(&cnt, 8, 1, fp);
      std::fwrite(e.bytes.data(), 1, e.bytes.size(), fp);
    }
    std::fclose(fp);
  }
};

}  // namespace kv
