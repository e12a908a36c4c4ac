// sfd_h5.hpp -- the reference's HDF5 state files from C++ without an HDF5
// library: saveStateFile / loadStateFile (SimulationRunner.cuh:99-178) over a
// minimal reader and writer of the subset of the format that libhdf5 writes
// with its default (earliest) settings:
// - version-0 superblock, 8-byte offsets and lengths;
// - version-1 object headers;
// - the root group as a symbol table (local heap, one B-tree leaf, one
//   symbol-table node);
// - contiguous datasets of little-endian doubles;
// - version-1 scalar attributes (double, int64, and bool as the FALSE/TRUE
//   enum over a signed byte, as HighFive and h5py store it).
// The byte layout is the one of superfluid_dynamics_gb300/h5io.py and files
// from either side open in the other; the encoding matches libhdf5's own, the
// subset h5py and HighFive read.  Header-only C++17,
// no CUDA; assumes a little-endian host (x86-64, aarch64).
#pragma once

#include <algorithm>
#include <complex>
#include <cstdint>
#include <cstring>
#include <fstream>
#include <iterator>
#include <map>
#include <stdexcept>
#include <string>
#include <utility>
#include <variant>
#include <vector>

namespace sfd {
namespace h5 {

using Attr = std::variant<double, long long, bool>;

struct Dataset {
  std::vector<uint64_t> shape;
  std::vector<double> data;  // row-major
};

namespace detail {

constexpr uint64_t kUndef = ~0ULL;
constexpr int kLeafK = 4, kInternalK = 16;

inline size_t pad8(size_t n) { return (n + 7) & ~size_t(7); }

template <typename T>
void put(std::string& b, T v) {
  b.append(reinterpret_cast<const char*>(&v), sizeof(T));
}
inline void zeros(std::string& b, size_t n) { b.append(n, '\0'); }
inline void pad_to8(std::string& b) { zeros(b, pad8(b.size()) - b.size()); }

inline std::string dtype_double() {
  std::string b = {'\x11', '\x20', '\x3f', '\x00'};
  put<uint32_t>(b, 8);
  put<uint16_t>(b, 0);
  put<uint16_t>(b, 64);
  b += {'\x34', '\x0b', '\x00', '\x34'};  // exponent at 52 (11 bits), mantissa at 0 (52 bits)
  put<uint32_t>(b, 1023);
  return b;
}
inline std::string dtype_int64() {
  std::string b = {'\x10', '\x08', '\x00', '\x00'};
  put<uint32_t>(b, 8);
  put<uint16_t>(b, 0);
  put<uint16_t>(b, 64);
  return b;
}
inline std::string dtype_bool() {
  std::string b = {'\x18', '\x02', '\x00', '\x00'};
  put<uint32_t>(b, 1);
  b += {'\x10', '\x08', '\x00', '\x00'};  // base: signed 8-bit integer
  put<uint32_t>(b, 1);
  put<uint16_t>(b, 0);
  put<uint16_t>(b, 8);
  std::string f = "FALSE", t = "TRUE";
  b += f;
  zeros(b, 8 - f.size());
  b += t;
  zeros(b, 8 - t.size());
  b += {'\x00', '\x01'};
  return b;
}
inline std::string dataspace(const std::vector<uint64_t>& shape, bool maxdims) {
  std::string b;
  put<uint8_t>(b, 1);
  put<uint8_t>(b, (uint8_t)shape.size());
  put<uint8_t>(b, (maxdims && !shape.empty()) ? 1 : 0);
  put<uint8_t>(b, 0);
  put<uint32_t>(b, 0);
  for (uint64_t d : shape) put<uint64_t>(b, d);
  if (maxdims && !shape.empty())
    for (uint64_t d : shape) put<uint64_t>(b, d);
  return b;
}
inline std::string message(uint16_t type, std::string body, uint8_t flags = 0) {
  pad_to8(body);
  std::string b;
  put<uint16_t>(b, type);
  put<uint16_t>(b, (uint16_t)body.size());
  put<uint8_t>(b, flags);
  zeros(b, 3);
  return b + body;
}
inline std::string object_header(const std::vector<std::string>& msgs) {
  std::string data;
  for (const auto& m : msgs) data += m;
  std::string b;
  put<uint8_t>(b, 1);
  put<uint8_t>(b, 0);
  put<uint16_t>(b, (uint16_t)msgs.size());
  put<uint32_t>(b, 1);
  put<uint32_t>(b, (uint32_t)data.size());
  zeros(b, 4);
  return b + data;
}
inline std::string attribute(const std::string& name, const Attr& v) {
  std::string dt, raw;
  if (std::holds_alternative<bool>(v)) {
    dt = dtype_bool();
    raw.push_back(std::get<bool>(v) ? '\x01' : '\x00');
  } else if (std::holds_alternative<long long>(v)) {
    dt = dtype_int64();
    put<int64_t>(raw, std::get<long long>(v));
  } else {
    dt = dtype_double();
    put<double>(raw, std::get<double>(v));
  }
  const std::string ds = dataspace({}, false);
  std::string nm = name;
  nm.push_back('\0');
  std::string b;
  put<uint8_t>(b, 1);
  put<uint8_t>(b, 0);
  put<uint16_t>(b, (uint16_t)nm.size());
  put<uint16_t>(b, (uint16_t)dt.size());
  put<uint16_t>(b, (uint16_t)ds.size());
  b += nm;
  zeros(b, pad8(nm.size()) - nm.size());
  b += dt;
  zeros(b, pad8(dt.size()) - dt.size());
  b += ds;
  zeros(b, pad8(ds.size()) - ds.size());
  return message(0x000C, b + raw);
}

struct Bytes {
  std::string b;
  template <typename T>
  T at(size_t off) const {
    if (off + sizeof(T) > b.size()) throw std::runtime_error("HDF5: read past the end of the file");
    T v;
    std::memcpy(&v, b.data() + off, sizeof(T));
    return v;
  }
  std::string cstr(size_t off) const {
    const size_t e = b.find('\0', off);
    if (e == std::string::npos) throw std::runtime_error("HDF5: unterminated name");
    return b.substr(off, e - off);
  }
};

struct Msg {
  uint16_t type;
  size_t body, size;
};
inline std::vector<Msg> messages(const Bytes& f, size_t addr) {
  if (f.at<uint8_t>(addr) != 1) throw std::runtime_error("HDF5: object header version not supported");
  const uint16_t n = f.at<uint16_t>(addr + 2);
  std::vector<std::pair<size_t, size_t>> chunks = {{addr + 16, f.at<uint32_t>(addr + 8)}};
  std::vector<Msg> out;
  for (size_t c = 0; c < chunks.size() && out.size() < n; ++c) {
    size_t p = chunks[c].first;
    const size_t end = p + chunks[c].second;
    while (p + 8 <= end && out.size() < n) {
      Msg m{f.at<uint16_t>(p), p + 8, f.at<uint16_t>(p + 2)};
      if (m.type == 0x0010) chunks.push_back({(size_t)f.at<uint64_t>(m.body), (size_t)f.at<uint64_t>(m.body + 8)});
      out.push_back(m);
      p += 8 + m.size;
    }
  }
  return out;
}
inline std::vector<uint64_t> read_dataspace(const Bytes& f, size_t p) {
  const uint8_t ver = f.at<uint8_t>(p), rank = f.at<uint8_t>(p + 1);
  const size_t base = p + (ver == 1 ? 8 : 4);
  std::vector<uint64_t> s(rank);
  for (int i = 0; i < rank; ++i) s[i] = f.at<uint64_t>(base + 8 * i);
  return s;
}

}  // namespace detail

// Write double datasets and root attributes.
inline void write(const std::string& path, const std::vector<std::pair<std::string, Dataset>>& datasets,
                  const std::vector<std::pair<std::string, Attr>>& attrs) {
  using namespace detail;
  if (datasets.empty() || datasets.size() > 2 * kLeafK)
    throw std::runtime_error("HDF5: between 1 and 8 datasets per file");
  std::string heap(8, '\0');
  std::vector<uint64_t> offs;
  for (const auto& d : datasets) {
    offs.push_back(heap.size());
    heap += d.first;
    heap.push_back('\0');
    pad_to8(heap);
  }
  std::vector<std::string> attr_msgs;
  size_t root_len = message(0x0011, std::string(16, '\0')).size();
  for (const auto& a : attrs) {
    attr_msgs.push_back(attribute(a.first, a.second));
    root_len += attr_msgs.back().size();
  }
  const size_t a_root = 96, a_btree = a_root + 16 + root_len;
  const size_t btree_size = 24 + (2 * kInternalK + 1) * 8 + 2 * kInternalK * 8;
  const size_t a_heap = a_btree + btree_size, a_heapdata = a_heap + 32, a_snod = a_heapdata + heap.size();
  const size_t snod_size = 8 + 2 * kLeafK * 40;
  auto header = [](const Dataset& d, uint64_t addr) {
    std::string lay;
    put<uint8_t>(lay, 3);
    put<uint8_t>(lay, 1);
    put<uint64_t>(lay, addr);
    put<uint64_t>(lay, (uint64_t)d.data.size() * 8);
    return object_header({message(0x0001, dataspace(d.shape, true)), message(0x0003, dtype_double(), 1),
                          message(0x0005, std::string("\x02\x02\x02\x01\x00\x00\x00\x00", 8), 1),
                          message(0x0008, lay)});
  };
  std::vector<size_t> hdr(datasets.size()), dat(datasets.size());
  size_t pos = a_snod + snod_size;
  for (size_t i = 0; i < datasets.size(); ++i) {
    uint64_t count = 1;
    for (uint64_t d : datasets[i].second.shape) count *= d;
    if (count != datasets[i].second.data.size()) throw std::runtime_error("HDF5: shape does not match the data");
    hdr[i] = pos;
    pos = pad8(pos + header(datasets[i].second, 0).size());
  }
  for (size_t i = 0; i < datasets.size(); ++i) {
    dat[i] = pos;
    pos = pad8(pos + datasets[i].second.data.size() * 8);
  }
  const size_t eof = pos;
  std::string file(eof, '\0');
  auto place = [&file](size_t at, const std::string& blob) { std::memcpy(&file[at], blob.data(), blob.size()); };
  // superblock
  std::string sb = std::string("\x89HDF\r\n\x1a\n", 8) + std::string("\x00\x00\x00\x00\x00\x08\x08\x00", 8);
  put<uint16_t>(sb, kLeafK);
  put<uint16_t>(sb, kInternalK);
  put<uint32_t>(sb, 0);
  for (uint64_t v : {uint64_t(0), kUndef, uint64_t(eof), kUndef, uint64_t(0), uint64_t(a_root)}) put<uint64_t>(sb, v);
  put<uint32_t>(sb, 1);
  put<uint32_t>(sb, 0);
  put<uint64_t>(sb, a_btree);
  put<uint64_t>(sb, a_heap);
  place(0, sb);
  // root group
  std::string st;
  put<uint64_t>(st, a_btree);
  put<uint64_t>(st, a_heap);
  std::vector<std::string> rmsgs = {message(0x0011, st)};
  rmsgs.insert(rmsgs.end(), attr_msgs.begin(), attr_msgs.end());
  place(a_root, object_header(rmsgs));
  // symbols in byte order of their names
  std::vector<size_t> order(datasets.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = i;
  std::sort(order.begin(), order.end(), [&](size_t a, size_t b) { return datasets[a].first < datasets[b].first; });
  std::string bt = "TREE";
  put<uint8_t>(bt, 0);
  put<uint8_t>(bt, 0);
  put<uint16_t>(bt, 1);
  put<uint64_t>(bt, kUndef);
  put<uint64_t>(bt, kUndef);
  put<uint64_t>(bt, 0);
  put<uint64_t>(bt, a_snod);
  put<uint64_t>(bt, offs[order.back()]);
  place(a_btree, bt);
  std::string hh = "HEAP";
  zeros(hh, 4);
  put<uint64_t>(hh, heap.size());
  put<uint64_t>(hh, 1);  // no free block
  put<uint64_t>(hh, a_heapdata);
  place(a_heap, hh);
  place(a_heapdata, heap);
  std::string sn = "SNOD";
  put<uint8_t>(sn, 1);
  put<uint8_t>(sn, 0);
  put<uint16_t>(sn, (uint16_t)datasets.size());
  for (size_t i : order) {
    put<uint64_t>(sn, offs[i]);
    put<uint64_t>(sn, hdr[i]);
    put<uint32_t>(sn, 0);
    put<uint32_t>(sn, 0);
    zeros(sn, 16);
  }
  place(a_snod, sn);
  for (size_t i = 0; i < datasets.size(); ++i) {
    place(hdr[i], header(datasets[i].second, dat[i]));
    if (!datasets[i].second.data.empty())
      std::memcpy(&file[dat[i]], datasets[i].second.data.data(), datasets[i].second.data.size() * 8);
  }
  std::ofstream out(path, std::ios::binary);
  if (!out) throw std::runtime_error("HDF5: cannot create " + path);
  out.write(file.data(), (std::streamsize)file.size());
  if (!out) throw std::runtime_error("HDF5: write failed for " + path);
}

// Read the double datasets and scalar root attributes of a file in the subset.
inline void read(const std::string& path, std::map<std::string, Dataset>& datasets,
                 std::map<std::string, Attr>& attrs) {
  using namespace detail;
  std::ifstream in(path, std::ios::binary);
  if (!in) throw std::runtime_error("HDF5: cannot open " + path);
  Bytes f{std::string((std::istreambuf_iterator<char>(in)), std::istreambuf_iterator<char>())};
  if (f.b.size() < 96 || f.b.compare(0, 8, std::string("\x89HDF\r\n\x1a\n", 8)) != 0)
    throw std::runtime_error("HDF5: " + path + " is not an HDF5 file");
  if (f.at<uint8_t>(8) != 0 || f.at<uint8_t>(13) != 8 || f.at<uint8_t>(14) != 8)
    throw std::runtime_error("HDF5: superblock version not supported");
  uint64_t bt = 0, hp = 0;
  for (const Msg& m : messages(f, f.at<uint64_t>(64))) {
    if (m.type == 0x0011) {
      bt = f.at<uint64_t>(m.body);
      hp = f.at<uint64_t>(m.body + 8);
    } else if (m.type == 0x000C) {
      const uint16_t nlen = f.at<uint16_t>(m.body + 2), dlen = f.at<uint16_t>(m.body + 4);
      const uint16_t slen = f.at<uint16_t>(m.body + 6);
      size_t p = m.body + 8;
      const std::string name = f.b.substr(p, nlen - 1);
      p += pad8(nlen);
      const size_t dt = p;
      p += pad8(dlen) + pad8(slen);
      const uint8_t cls = f.at<uint8_t>(dt) & 0x0F;
      if (cls == 1) attrs[name] = f.at<double>(p);
      else if (cls == 0) attrs[name] = (long long)f.at<int64_t>(p);
      else if (cls == 8) attrs[name] = f.at<int8_t>(p) != 0;
    }
  }
  if (!bt) throw std::runtime_error("HDF5: root group is not a symbol-table group");
  const uint64_t hdata = f.at<uint64_t>(hp + 24);
  if (f.b.compare(bt, 4, "TREE") != 0) throw std::runtime_error("HDF5: bad B-tree node");
  if (f.at<uint8_t>(bt + 5) != 0) throw std::runtime_error("HDF5: multi-level group B-trees not supported");
  for (uint16_t c = 0; c < f.at<uint16_t>(bt + 6); ++c) {
    const uint64_t snod = f.at<uint64_t>(bt + 24 + 8 + 16 * c);
    if (f.b.compare(snod, 4, "SNOD") != 0) throw std::runtime_error("HDF5: bad symbol-table node");
    for (uint16_t i = 0; i < f.at<uint16_t>(snod + 6); ++i) {
      const size_t e = snod + 8 + 40 * i;
      const std::string name = f.cstr(hdata + f.at<uint64_t>(e));
      Dataset d;
      uint64_t addr = kUndef;
      bool is_double = false;
      for (const Msg& m : messages(f, f.at<uint64_t>(e + 8))) {
        if (m.type == 0x0001) d.shape = read_dataspace(f, m.body);
        else if (m.type == 0x0003) is_double = (f.at<uint8_t>(m.body) & 0x0F) == 1 && f.at<uint32_t>(m.body + 4) == 8;
        else if (m.type == 0x0008) {
          if (f.at<uint8_t>(m.body) != 3 || f.at<uint8_t>(m.body + 1) != 1)
            throw std::runtime_error("HDF5: dataset " + name + ": only contiguous layout is supported");
          addr = f.at<uint64_t>(m.body + 2);
        }
      }
      if (!is_double) continue;  // not a double dataset: outside this reader
      uint64_t count = 1;
      for (uint64_t s : d.shape) {
        if (s != 0 && count > UINT64_MAX / s) throw std::runtime_error("HDF5: dataset " + name + ": shape overflows");
        count *= s;
      }
      // checked before the allocation, so a malformed shape cannot ask for more than the file holds
      if (addr != kUndef && count && (addr > f.b.size() || count > (f.b.size() - addr) / 8))
        throw std::runtime_error("HDF5: dataset " + name + " runs past the end of the file");
      d.data.resize(count);
      if (addr != kUndef && count) std::memcpy(d.data.data(), f.b.data() + addr, count * 8);
      datasets[name] = std::move(d);
    }
  }
}

}  // namespace h5

// saveStateFile (SimulationRunner.cuh:144-178): `interface` (N x 2: Re Z, Im Z),
// `potential` (N), root attributes rho, kappa, U, depth, initial_amplitude, rhs.
inline int saveStateFile(const std::string& path, const std::vector<std::complex<double>>& Z,
                         const std::vector<double>& phi, size_t N, double rho, double kappa, double U, double depth,
                         double initial_amplitude, bool rhs = false) {
  if (Z.size() != N || phi.size() != N) throw std::runtime_error("saveStateFile: Z and phi must hold N values");
  h5::Dataset itf{{N, 2}, std::vector<double>(2 * N)}, pot{{N}, phi};
  for (size_t i = 0; i < N; ++i) {
    itf.data[2 * i] = Z[i].real();
    itf.data[2 * i + 1] = Z[i].imag();
  }
  h5::write(path, {{"interface", itf}, {"potential", pot}},
            {{"rho", rho}, {"kappa", kappa}, {"U", U}, {"depth", depth}, {"initial_amplitude", initial_amplitude},
             {"rhs", rhs}});
  return 0;
}

// loadStateFile (SimulationRunner.cuh:99-142): Z = x + i scaleY y from
// `interface`, phi from `potential`, with the reference's shape checks.
inline int loadStateFile(const std::string& path, std::vector<std::complex<double>>& Z, std::vector<double>& phi,
                         size_t N, double scaleY = 1.0) {
  std::map<std::string, h5::Dataset> ds;
  std::map<std::string, h5::Attr> at;
  h5::read(path, ds, at);
  if (!ds.count("interface") || !ds.count("potential"))
    throw std::runtime_error("the file must hold the datasets 'interface' and 'potential'");
  const auto& itf = ds["interface"];
  const auto& dims = itf.shape;
  if (dims.size() != 2 || dims[1] != 2 || dims[0] != N) {
    const std::string want = "Interface must have shape (" + std::to_string(N) + ", 2), instead it has ";
    if (dims.size() == 1) throw std::runtime_error(want + "(" + std::to_string(dims[0]) + ",)");
    if (dims.size() == 2)
      throw std::runtime_error(want + "(" + std::to_string(dims[0]) + ", " + std::to_string(dims[1]) + ")");
    throw std::runtime_error(want + "a higher dimensionality than 2 (" + std::to_string(dims.size()) + ")!");
  }
  if (ds["potential"].shape.empty()) throw std::runtime_error("potential dataset is empty.");
  phi = ds["potential"].data;
  Z.resize(N);
  for (size_t i = 0; i < N; ++i) Z[i] = {itf.data[2 * i], scaleY * itf.data[2 * i + 1]};
  return 0;
}

}  // namespace sfd
