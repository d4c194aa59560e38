// netcdf_io.cpp -- the on-disk formats of jif3D's data and models: a NetCDF
// reader and writer with no NetCDF or HDF5 library underneath.
//
// Reading: NetCDF classic files (CDF-1, CDF-2 64-bit offset, CDF-5) and
// netCDF-4 files, i.e. HDF5 files in the shape the netCDF-4 library gives
// them: superblock 0-3, object headers 1 and 2, groups with compact links
// (link messages in the object header) or an old-style symbol table,
// contiguous or compact datasets of IEEE floats or two's-complement integers,
// fixed-length string attributes.  Chunked (compressed) datasets and dense
// link storage are reported as unsupported.  netCDF-4 dimensions without a
// coordinate variable are HDF5 "dimension scale" datasets; they are read as
// dimensions only.
//
// Writing: CDF-2 (64-bit offset) classic files, which every NetCDF library
// reads -- jif3D's netCDF-C++ reads them as it reads its own netCDF-4 files.
//
// Host code only (no CUDA): the C ABI entry points are j3g_nc_* in
// include/jif3d_gb300.h.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/jif3d_gb300.h"

namespace {

thread_local std::string g_nc_error;

struct NcError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// one variable, its values converted to double
struct Var {
  std::string name;
  std::vector<long long> shape;
  std::vector<std::string> dims;  // dimension names (classic files)
  int type = J3G_NC_DOUBLE;
  std::vector<double> values;
  std::map<std::string, std::string> text_atts;
  std::map<std::string, std::vector<double>> num_atts;
};

struct File {
  std::vector<Var> vars;
  std::vector<std::pair<std::string, long long>> dims;
  std::map<std::string, std::string> text_atts;  // global
  std::map<std::string, std::vector<double>> num_atts;
  int format = 0;  // 1, 2, 5 classic; 4 HDF5
  const Var *find(const std::string &n) const {
    for (const Var &v : vars)
      if (v.name == n) return &v;
    return nullptr;
  }
};

std::vector<uint8_t> read_all(const char *path) {
  FILE *f = std::fopen(path, "rb");
  if (!f) throw NcError(std::string("cannot open ") + path);
  std::vector<uint8_t> d;
  uint8_t buf[1 << 16];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof buf, f)) > 0) d.insert(d.end(), buf, buf + n);
  std::fclose(f);
  return d;
}

// ---------------------------------------------------------------------------
// NetCDF classic (big-endian, the format of the NetCDF User's Guide, "File
// Format Specification")
class ClassicReader {
 public:
  explicit ClassicReader(const std::vector<uint8_t> &d) : d_(d) {}

  File parse() {
    File f;
    if (d_.size() < 4 || std::memcmp(d_.data(), "CDF", 3) != 0) throw NcError("not a CDF file");
    version_ = d_[3];
    if (version_ != 1 && version_ != 2 && version_ != 5)
      throw NcError("unknown CDF version " + std::to_string(version_));
    f.format = version_;
    pos_ = 4;
    const uint64_t numrecs = count();
    // dimensions
    uint32_t tag = u32();
    const uint64_t ndims = count();
    if (tag != 0x0A && !(tag == 0 && ndims == 0)) throw NcError("bad dimension list");
    int recdim = -1;
    for (uint64_t i = 0; i < ndims; ++i) {
      std::string name = str();
      const uint64_t len = count();
      if (len == 0) recdim = (int)i;
      f.dims.push_back({name, len == 0 ? (long long)numrecs : (long long)len});
    }
    atts(f.text_atts, f.num_atts);
    tag = u32();
    const uint64_t nvars = count();
    if (tag != 0x0B && !(tag == 0 && nvars == 0)) throw NcError("bad variable list");
    struct Layout {
      int type;
      uint64_t vsize, begin;
      bool rec;
    };
    std::vector<Layout> lay;
    for (uint64_t i = 0; i < nvars; ++i) {
      Var v;
      v.name = str();
      const uint64_t nd = count();
      bool rec = false;
      for (uint64_t k = 0; k < nd; ++k) {
        const uint64_t id = count();
        if (id >= f.dims.size()) throw NcError("bad dimension id in " + v.name);
        if (k == 0 && (int)id == recdim) rec = true;
        v.dims.push_back(f.dims[id].first);
        v.shape.push_back(f.dims[id].second);
      }
      atts(v.text_atts, v.num_atts);
      v.type = (int)u32();
      const uint64_t vsize = count();
      const uint64_t begin = version_ == 1 ? u32() : u64();
      lay.push_back({v.type, vsize, begin, rec});
      f.vars.push_back(std::move(v));
    }
    // the record size: the record variables' vsizes, in order
    uint64_t recsize = 0;
    int nrecvars = 0;
    for (auto &l : lay)
      if (l.rec) recsize += l.vsize, ++nrecvars;
    for (size_t i = 0; i < f.vars.size(); ++i) {
      Var &v = f.vars[i];
      long long n = 1;
      for (long long s : v.shape) n *= s;
      v.values.resize((size_t)n);
      const int esz = type_size(lay[i].type);
      if (!lay[i].rec) {
        for (long long k = 0; k < n; ++k) v.values[k] = value(lay[i].type, lay[i].begin + k * esz);
      } else {
        // one record's slab per record; a lone record variable is not padded
        long long per = n / std::max<long long>(1, v.shape[0]);
        const uint64_t stride = nrecvars == 1 ? (uint64_t)(per * esz) : recsize;
        for (long long r = 0; r < v.shape[0]; ++r)
          for (long long k = 0; k < per; ++k)
            v.values[r * per + k] = value(lay[i].type, lay[i].begin + r * stride + k * esz);
      }
      v.type = lay[i].type;
    }
    return f;
  }

 private:
  void need(uint64_t n) const {
    if (pos_ + n > d_.size()) throw NcError("truncated CDF file");
  }
  uint32_t u32() {
    need(4);
    uint32_t v = 0;
    for (int i = 0; i < 4; ++i) v = v << 8 | d_[pos_ + i];
    pos_ += 4;
    return v;
  }
  uint64_t u64() {
    const uint64_t hi = u32();
    return hi << 32 | u32();
  }
  uint64_t count() { return version_ == 5 ? u64() : u32(); }
  std::string str() {
    const uint64_t n = count();
    need(n);
    std::string s(reinterpret_cast<const char *>(d_.data() + pos_), n);
    pos_ += (n + 3) / 4 * 4;
    return s;
  }
  static int type_size(int t) {
    switch (t) {
      case 1: case 2: case 7: return 1;
      case 3: case 8: return 2;
      case 4: case 5: case 9: return 4;
      case 6: case 10: case 11: return 8;
    }
    throw NcError("unknown NetCDF type " + std::to_string(t));
  }
  double value(int t, uint64_t off) const {
    const int n = type_size(t);
    if (off + n > d_.size()) throw NcError("variable data beyond the end of the file");
    uint64_t bits = 0;
    for (int i = 0; i < n; ++i) bits = bits << 8 | d_[off + i];
    switch (t) {
      case 1: return (double)(int8_t)bits;
      case 2: case 7: return (double)(uint8_t)bits;
      case 3: return (double)(int16_t)bits;
      case 8: return (double)(uint16_t)bits;
      case 4: return (double)(int32_t)bits;
      case 9: return (double)(uint32_t)bits;
      case 10: return (double)(int64_t)bits;
      case 11: return (double)bits;
      case 5: {
        const uint32_t b = (uint32_t)bits;
        float x;
        std::memcpy(&x, &b, 4);
        return x;
      }
      default: {
        double x;
        std::memcpy(&x, &bits, 8);
        return x;
      }
    }
  }
  void atts(std::map<std::string, std::string> &text, std::map<std::string, std::vector<double>> &num) {
    const uint32_t tag = u32();
    const uint64_t n = count();
    if (tag != 0x0C && !(tag == 0 && n == 0)) throw NcError("bad attribute list");
    for (uint64_t i = 0; i < n; ++i) {
      std::string name = str();
      const int t = (int)u32();
      const uint64_t ne = count();
      const int esz = type_size(t);
      need(ne * esz);
      if (t == 2) {
        std::string s(reinterpret_cast<const char *>(d_.data() + pos_), ne);
        s.erase(std::find(s.begin(), s.end(), '\0'), s.end());
        text[name] = s;
      } else {
        std::vector<double> v(ne);
        for (uint64_t k = 0; k < ne; ++k) v[k] = value(t, pos_ + k * esz);
        num[name] = v;
      }
      pos_ += (ne * esz + 3) / 4 * 4;
    }
  }

  const std::vector<uint8_t> &d_;
  uint64_t pos_ = 0;
  int version_ = 1;
};

// ---------------------------------------------------------------------------
// HDF5 (the public HDF5 File Format Specification, version 3.0), the subset
// that netCDF-4 files of jif3D's data and models use
class H5Reader {
 public:
  explicit H5Reader(const std::vector<uint8_t> &d) : d_(d) {}

  File parse() {
    static const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    // the superblock may sit at 0, 512, 1024, ... (a user block before it)
    uint64_t sb = UINT64_MAX;
    for (uint64_t off = 0; off + 8 <= d_.size(); off = off ? off * 2 : 512)
      if (std::memcmp(d_.data() + off, sig, 8) == 0) {
        sb = off;
        break;
      }
    if (sb == UINT64_MAX) throw NcError("not an HDF5 file");
    const int ver = byte(sb + 8);
    uint64_t root = 0;
    if (ver == 0 || ver == 1) {
      so_ = byte(sb + 13);
      sl_ = byte(sb + 14);
      uint64_t p = sb + 24 + (ver == 1 ? 4 : 0);
      base_ = uint(p, so_);
      p += 4 * so_;          // base, free space, end of file, driver info
      root = uint(p + so_, so_);  // root symbol table entry: name offset, header
    } else if (ver == 2 || ver == 3) {
      so_ = byte(sb + 9);
      sl_ = byte(sb + 10);
      base_ = uint(sb + 12, so_);
      root = uint(sb + 12 + 3 * so_, so_);  // base, extension, end of file, root
    } else {
      throw NcError("unsupported HDF5 superblock version " + std::to_string(ver));
    }
    if (so_ != 8 && so_ != 4) throw NcError("unsupported HDF5 offset size");
    File f;
    f.format = 4;
    Object o = object(root);
    for (auto &a : o.text) f.text_atts[a.first] = a.second;
    for (auto &a : o.num) f.num_atts[a.first] = a.second;
    for (auto &l : links(o)) {
      Object c = object(l.second);
      if (!c.is_dataset) continue;  // sub-groups: not used by jif3D files
      Var v;
      v.name = l.first;
      v.shape = c.shape;
      v.type = c.nc_type;
      v.values = c.values;
      v.text_atts = c.text;
      v.num_atts = c.num;
      const auto cls = c.text.find("CLASS");
      const auto nm = c.text.find("NAME");
      const bool scale = cls != c.text.end() && cls->second == "DIMENSION_SCALE";
      if (scale) f.dims.push_back({v.name, v.shape.empty() ? 1 : v.shape[0]});
      // a dimension without a coordinate variable is not a variable
      if (scale && nm != c.text.end() &&
          nm->second.find("This is a netCDF dimension but not a netCDF variable") == 0)
        continue;
      // netCDF-4 bookkeeping attributes are not the variable's own
      for (const char *k : {"CLASS", "NAME", "_Netcdf4Dimid", "_Netcdf4Coordinates"}) {
        v.text_atts.erase(k);
        v.num_atts.erase(k);
      }
      f.vars.push_back(std::move(v));
    }
    f.text_atts.erase("_NCProperties");
    f.num_atts.erase("_NCProperties");
    return f;
  }

 private:
  struct Object {
    std::vector<std::pair<std::string, uint64_t>> links;
    bool has_link_info = false, dense = false, symtab = false;
    uint64_t btree = 0, heap = 0;
    bool is_dataset = false;
    std::vector<long long> shape;
    int nc_type = J3G_NC_DOUBLE;
    std::vector<double> values;
    std::map<std::string, std::string> text;
    std::map<std::string, std::vector<double>> num;
    // raw pieces of a dataset
    bool have_space = false, have_type = false, have_layout = false, null_space = false;
    uint8_t hflags = 0;  // version-2 object header flags
    std::vector<uint8_t> type_msg;
    int layout_class = -1;
    uint64_t data_addr = 0, data_size = 0;
    std::vector<uint8_t> compact;
  };

  uint8_t byte(uint64_t p) const {
    if (p >= d_.size()) throw NcError("truncated HDF5 file");
    return d_[p];
  }
  uint64_t uint(uint64_t p, int n) const {
    if (p + n > d_.size()) throw NcError("truncated HDF5 file");
    uint64_t v = 0;
    for (int i = n - 1; i >= 0; --i) v = v << 8 | d_[p + i];
    return v;
  }
  bool undefined(uint64_t a) const { return so_ == 8 ? a == UINT64_MAX : a == 0xFFFFFFFFull; }
  uint64_t addr(uint64_t a) const { return base_ + a; }

  // an object header (version 1 or 2) and its continuation blocks
  Object object(uint64_t a) {
    Object o;
    const uint64_t p = addr(a);
    if (p + 4 <= d_.size() && std::memcmp(d_.data() + p, "OHDR", 4) == 0) {
      const uint8_t flags = byte(p + 5);
      uint64_t q = p + 6;
      if (flags & 0x20) q += 16;  // times
      if (flags & 0x10) q += 4;   // attribute phase change
      const int szb = 1 << (flags & 3);
      const uint64_t size0 = uint(q, szb);
      q += szb;
      o.hflags = flags;
      messages_v2(o, q, q + size0);
    } else {
      if (byte(p) != 1) throw NcError("unsupported HDF5 object header version");
      const uint64_t size0 = uint(p + 8, 4);
      messages_v1(o, p + 16, p + 16 + size0);
    }
    finish(o);
    return o;
  }
  void messages_v2(Object &o, uint64_t q, uint64_t end) {
    while (q + 4 <= end) {
      const int type = byte(q);
      const uint64_t size = uint(q + 1, 2);
      const uint8_t mflags = byte(q + 3);
      q += 4 + ((o.hflags & 0x04) ? 2 : 0);
      if (q + size > end) break;
      message(o, type, q, size, mflags, true);
      q += size;
    }
  }
  void messages_v1(Object &o, uint64_t q, uint64_t end) {
    while (q + 8 <= end) {
      const int type = (int)uint(q, 2);
      const uint64_t size = uint(q + 2, 2);
      const uint8_t mflags = byte(q + 4);
      q += 8;
      if (q + size > end) break;
      message(o, type, q, size, mflags, false);
      q += size;
    }
  }
  void message(Object &o, int type, uint64_t q, uint64_t size, uint8_t mflags, bool v2) {
    if (mflags & 0x02) {  // a shared message: only a few kinds would be, none here
      throw NcError("shared HDF5 object header messages are not supported");
    }
    switch (type) {
      case 0x01: dataspace(o, q); break;
      case 0x03:
        o.type_msg.assign(d_.begin() + q, d_.begin() + q + size);
        o.have_type = true;
        break;
      case 0x08: layout(o, q); break;
      case 0x0C: attribute(o, q, size); break;
      case 0x06: link(o, q); break;
      case 0x02: {  // link info: dense storage if a fractal heap exists
        o.has_link_info = true;
        const uint8_t fl = byte(q + 1);
        const uint64_t heap = uint(q + 2 + ((fl & 1) ? 8 : 0), so_);
        if (!undefined(heap)) o.dense = true;
        break;
      }
      case 0x11:  // old-style group: symbol table (v1 B-tree + local heap)
        o.symtab = true;
        o.btree = uint(q, so_);
        o.heap = uint(q + so_, so_);
        break;
      case 0x10: {  // continuation block
        const uint64_t off = addr(uint(q, so_));
        const uint64_t len = uint(q + so_, sl_);
        if (v2) {
          if (off + 4 > d_.size() || std::memcmp(d_.data() + off, "OCHK", 4) != 0)
            throw NcError("bad HDF5 continuation block");
          messages_v2(o, off + 4, off + len - 4);
        } else {
          messages_v1(o, off, off + len);
        }
        break;
      }
      default: break;  // fill value, modification time, group info, ... not needed
    }
  }
  void dataspace(Object &o, uint64_t q) {
    const int ver = byte(q);
    const int rank = byte(q + 1);
    uint64_t p;
    if (ver == 1) {
      p = q + 8;
    } else if (ver == 2) {
      p = q + 4;
      if (byte(q + 3) == 2) o.null_space = true;
    } else {
      throw NcError("unsupported HDF5 dataspace version");
    }
    o.shape.clear();
    for (int i = 0; i < rank; ++i) o.shape.push_back((long long)uint(p + (uint64_t)i * sl_, sl_));
    o.have_space = true;
  }
  void layout(Object &o, uint64_t q) {
    const int ver = byte(q);
    if (ver == 3 || ver == 4) {
      o.layout_class = byte(q + 1);
      if (o.layout_class == 0) {
        const uint64_t n = uint(q + 2, 2);
        o.compact.assign(d_.begin() + q + 4, d_.begin() + q + 4 + n);
      } else if (o.layout_class == 1) {
        o.data_addr = uint(q + 2, so_);
        o.data_size = uint(q + 2 + so_, sl_);
      }
    } else if (ver == 1 || ver == 2) {
      const int rank = byte(q + 1);
      o.layout_class = byte(q + 2);
      uint64_t p = q + 8;
      if (o.layout_class != 0) o.data_addr = uint(p, so_), p += so_;
      p += 4ull * rank;
      if (o.layout_class == 0) {
        const uint64_t n = uint(p, 4);
        o.compact.assign(d_.begin() + p + 4, d_.begin() + p + 4 + n);
      }
    } else {
      throw NcError("unsupported HDF5 layout version");
    }
    o.have_layout = true;
  }
  // converts n elements of an HDF5 datatype at src to doubles; false if the
  // type is not a number
  bool convert(const std::vector<uint8_t> &tm, const uint8_t *src, size_t n, std::vector<double> &out,
               int *nc_type) const {
    if (tm.size() < 8) return false;
    const int cls = tm[0] & 0x0F;
    const uint8_t b0 = tm[1];
    const uint32_t size = tm[4] | tm[5] << 8 | tm[6] << 16 | (uint32_t)tm[7] << 24;
    const bool big = b0 & 1;
    if (cls != 0 && cls != 1) return false;
    if (size != 1 && size != 2 && size != 4 && size != 8) return false;
    out.resize(n);
    for (size_t i = 0; i < n; ++i) {
      uint64_t bits = 0;
      const uint8_t *e = src + i * size;
      for (uint32_t k = 0; k < size; ++k) bits |= (uint64_t)e[big ? size - 1 - k : k] << (8 * k);
      if (cls == 1) {
        if (size == 8) {
          std::memcpy(&out[i], &bits, 8);
        } else if (size == 4) {
          const uint32_t b = (uint32_t)bits;
          float x;
          std::memcpy(&x, &b, 4);
          out[i] = x;
        } else {
          return false;
        }
      } else {
        const bool sgn = b0 & 0x08;
        const int shift = 64 - 8 * (int)size;
        out[i] = sgn ? (double)((int64_t)(bits << shift) >> shift) : (double)bits;
      }
    }
    if (nc_type) {
      if (cls == 1) *nc_type = size == 8 ? J3G_NC_DOUBLE : J3G_NC_FLOAT;
      else *nc_type = size == 4 ? J3G_NC_INT : (size == 2 ? J3G_NC_SHORT : J3G_NC_BYTE);
    }
    return true;
  }
  void attribute(Object &o, uint64_t q, uint64_t size) {
    const int ver = byte(q);
    const uint64_t nlen = uint(q + 2, 2), tlen = uint(q + 4, 2), slen = uint(q + 6, 2);
    uint64_t p = q + 8 + (ver == 3 ? 1 : 0);
    auto pad = [&](uint64_t n) { return ver == 1 ? (n + 7) / 8 * 8 : n; };
    std::string name(reinterpret_cast<const char *>(d_.data() + p), nlen);
    name.erase(std::find(name.begin(), name.end(), '\0'), name.end());
    p += pad(nlen);
    const uint64_t tp = p;
    p += pad(tlen);
    Object space;
    dataspace(space, p);
    p += pad(slen);
    long long n = 1;
    for (long long s : space.shape) n *= s;
    if (p > q + size) return;
    std::vector<uint8_t> tm(d_.begin() + tp, d_.begin() + tp + tlen);
    const int cls = tm.empty() ? -1 : (tm[0] & 0x0F);
    if (cls == 3) {  // fixed-length string
      const uint32_t sz = tm[4] | tm[5] << 8 | tm[6] << 16 | (uint32_t)tm[7] << 24;
      const uint64_t total = (uint64_t)sz * (uint64_t)std::max<long long>(1, n);
      if (p + total > d_.size()) return;
      std::string s(reinterpret_cast<const char *>(d_.data() + p), total);
      s.erase(std::find(s.begin(), s.end(), '\0'), s.end());
      while (!s.empty() && s.back() == ' ' && sz > 1 && s.size() == total) s.pop_back();
      o.text[name] = s;
    } else if (cls == 0 || cls == 1) {
      const uint32_t sz = tm[4] | tm[5] << 8 | tm[6] << 16 | (uint32_t)tm[7] << 24;
      if (p + (uint64_t)sz * n > d_.size()) return;
      std::vector<double> v;
      if (convert(tm, d_.data() + p, (size_t)n, v, nullptr)) o.num[name] = v;
    }
    // variable-length (references, vlen strings): not needed for jif3D files
  }
  void link(Object &o, uint64_t q) {
    const uint8_t fl = byte(q + 1);
    uint64_t p = q + 2;
    int ltype = 0;
    if (fl & 0x08) ltype = byte(p++);
    if (fl & 0x04) p += 8;
    if (fl & 0x10) p += 1;
    const int lsz = 1 << (fl & 3);
    const uint64_t nlen = uint(p, lsz);
    p += lsz;
    std::string name(reinterpret_cast<const char *>(d_.data() + p), nlen);
    p += nlen;
    if (ltype == 0) o.links.push_back({name, uint(p, so_)});
  }
  // old-style group members: v1 B-tree of symbol nodes, names in a local heap
  void symbol_table(Object &o) {
    const uint64_t hp = addr(o.heap);
    if (hp + 8 > d_.size() || std::memcmp(d_.data() + hp, "HEAP", 4) != 0)
      throw NcError("bad HDF5 local heap");
    const uint64_t heap_data = addr(uint(hp + 8 + 2 * sl_, so_));
    std::vector<uint64_t> todo{addr(o.btree)};
    while (!todo.empty()) {
      const uint64_t t = todo.back();
      todo.pop_back();
      if (std::memcmp(d_.data() + t, "TREE", 4) != 0) throw NcError("bad HDF5 B-tree node");
      const int level = byte(t + 5);
      const uint64_t used = uint(t + 6, 2);
      uint64_t p = t + 8 + 2 * so_;  // left and right siblings
      for (uint64_t i = 0; i < used; ++i) {
        p += sl_;  // key
        const uint64_t child = addr(uint(p, so_));
        p += so_;
        if (level > 0) {
          todo.push_back(child);
          continue;
        }
        if (std::memcmp(d_.data() + child, "SNOD", 4) != 0) throw NcError("bad HDF5 symbol node");
        const uint64_t nsym = uint(child + 6, 2);
        uint64_t e = child + 8;
        for (uint64_t k = 0; k < nsym; ++k, e += 2 * so_ + 24) {
          const uint64_t noff = uint(e, so_);
          const char *nm = reinterpret_cast<const char *>(d_.data() + heap_data + noff);
          o.links.push_back({std::string(nm), uint(e + so_, so_)});
        }
      }
    }
  }
  std::vector<std::pair<std::string, uint64_t>> links(Object &o) {
    if (o.dense) throw NcError("HDF5 groups with dense link storage are not supported");
    if (o.symtab) symbol_table(o);
    return o.links;
  }
  void finish(Object &o) {
    if (!(o.have_space && o.have_type && o.have_layout)) return;
    o.is_dataset = true;
    long long n = 1;
    for (long long s : o.shape) n *= s;
    if (o.null_space) n = 0;
    const uint32_t esz = o.type_msg.size() >= 8 ? (o.type_msg[4] | o.type_msg[5] << 8 |
                                                   o.type_msg[6] << 16 |
                                                   (uint32_t)o.type_msg[7] << 24)
                                                : 0;
    const uint64_t bytes = (uint64_t)n * esz;
    std::vector<uint8_t> raw;
    if (o.layout_class == 0) {
      raw = o.compact;
    } else if (o.layout_class == 1) {
      if (undefined(o.data_addr)) {
        raw.assign(bytes, 0);  // never written: the fill value 0
      } else {
        const uint64_t p = addr(o.data_addr);
        if (p + bytes > d_.size()) throw NcError("HDF5 dataset beyond the end of the file");
        raw.assign(d_.begin() + p, d_.begin() + p + bytes);
      }
    } else {
      throw NcError("chunked HDF5 datasets are not supported (write the file without "
                    "chunking or compression)");
    }
    if (raw.size() < bytes) throw NcError("short HDF5 dataset");
    std::vector<double> v;
    if (!convert(o.type_msg, raw.data(), (size_t)n, v, &o.nc_type)) {
      o.is_dataset = false;  // not a numeric variable (strings, references)
      return;
    }
    o.values = std::move(v);
  }

  const std::vector<uint8_t> &d_;
  int so_ = 8, sl_ = 8;
  uint64_t base_ = 0;
};

// ---------------------------------------------------------------------------
// CDF-2 writer
struct Writer {
  std::string path;
  std::vector<std::pair<std::string, long long>> dims;
  struct WVar {
    std::string name;
    int type;
    std::vector<int> dimids;
    std::vector<std::pair<std::string, std::string>> atts;
    std::vector<double> values;
    bool put = false;
  };
  std::vector<WVar> vars;
  std::vector<std::pair<std::string, std::string>> gatts;

  WVar *find(const std::string &n) {
    for (WVar &v : vars)
      if (v.name == n) return &v;
    return nullptr;
  }
  static void be32(std::vector<uint8_t> &o, uint32_t v) {
    for (int i = 3; i >= 0; --i) o.push_back((uint8_t)(v >> (8 * i)));
  }
  static void be64(std::vector<uint8_t> &o, uint64_t v) {
    be32(o, (uint32_t)(v >> 32));
    be32(o, (uint32_t)v);
  }
  static void name(std::vector<uint8_t> &o, const std::string &s) {
    be32(o, (uint32_t)s.size());
    o.insert(o.end(), s.begin(), s.end());
    while (o.size() % 4) o.push_back(0);
  }
  static void att_list(std::vector<uint8_t> &o,
                       const std::vector<std::pair<std::string, std::string>> &a) {
    if (a.empty()) {
      be32(o, 0), be32(o, 0);
      return;
    }
    be32(o, 0x0C);
    be32(o, (uint32_t)a.size());
    for (auto &x : a) {
      name(o, x.first);
      be32(o, J3G_NC_CHAR);
      be32(o, (uint32_t)x.second.size());
      o.insert(o.end(), x.second.begin(), x.second.end());
      while (o.size() % 4) o.push_back(0);
    }
  }
  static int esize(int t) { return t == J3G_NC_DOUBLE ? 8 : 4; }
  long long count(const WVar &v) const {
    long long n = 1;
    for (int d : v.dimids) n *= dims[d].second;
    return n;
  }
  void write() {
    for (auto &v : vars)
      if (!v.put) throw NcError("variable " + v.name + " was defined but not written");
    // the header with placeholder offsets, then the data
    auto header = [&](const std::vector<uint64_t> &begins) {
      std::vector<uint8_t> o = {'C', 'D', 'F', 2};
      be32(o, 0);  // numrecs
      if (dims.empty()) {
        be32(o, 0), be32(o, 0);
      } else {
        be32(o, 0x0A);
        be32(o, (uint32_t)dims.size());
        for (auto &d : dims) name(o, d.first), be32(o, (uint32_t)d.second);
      }
      att_list(o, gatts);
      if (vars.empty()) {
        be32(o, 0), be32(o, 0);
      } else {
        be32(o, 0x0B);
        be32(o, (uint32_t)vars.size());
        for (size_t i = 0; i < vars.size(); ++i) {
          const WVar &v = vars[i];
          name(o, v.name);
          be32(o, (uint32_t)v.dimids.size());
          for (int d : v.dimids) be32(o, (uint32_t)d);
          att_list(o, v.atts);
          be32(o, (uint32_t)v.type);
          const uint64_t vs = (uint64_t)count(v) * esize(v.type);
          be32(o, (uint32_t)std::min<uint64_t>((vs + 3) / 4 * 4, 0xFFFFFFFFull));
          be64(o, begins.empty() ? 0 : begins[i]);
        }
      }
      return o;
    };
    std::vector<uint64_t> begins;
    uint64_t off = header({}).size();
    for (auto &v : vars) {
      begins.push_back(off);
      off += ((uint64_t)count(v) * esize(v.type) + 3) / 4 * 4;
    }
    std::vector<uint8_t> o = header(begins);
    for (auto &v : vars) {
      for (double x : v.values) {
        if (v.type == J3G_NC_DOUBLE) {
          uint64_t b;
          std::memcpy(&b, &x, 8);
          be64(o, b);
        } else if (v.type == J3G_NC_FLOAT) {
          const float f = (float)x;
          uint32_t b;
          std::memcpy(&b, &f, 4);
          be32(o, b);
        } else {
          be32(o, (uint32_t)(int32_t)x);
        }
      }
      while (o.size() % 4) o.push_back(0);
    }
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) throw NcError("cannot create " + path);
    const size_t w = std::fwrite(o.data(), 1, o.size(), f);
    const int c = std::fclose(f);
    if (w != o.size() || c != 0) throw NcError("cannot write " + path);
  }
};

int fail(const std::string &msg) {
  g_nc_error = msg;
  return J3G_ERR_ARG;
}

}  // namespace

struct j3g_ncfile {
  File f;
};
struct j3g_ncwriter {
  Writer w;
};

extern "C" {

const char *j3g_nc_last_error(void) { return g_nc_error.c_str(); }

int j3g_nc_open(const char *path, j3g_ncfile **file) {
  if (!path || !file) return fail("null argument");
  *file = nullptr;
  try {
    const std::vector<uint8_t> d = read_all(path);
    auto h = std::make_unique<j3g_ncfile>();
    if (d.size() >= 4 && std::memcmp(d.data(), "CDF", 3) == 0)
      h->f = ClassicReader(d).parse();
    else
      h->f = H5Reader(d).parse();
    *file = h.release();
    return J3G_OK;
  } catch (const std::exception &e) {
    return fail(std::string(path) + ": " + e.what());
  }
}

int j3g_nc_close(j3g_ncfile *file) {
  delete file;
  return J3G_OK;
}

int j3g_nc_format(const j3g_ncfile *file, int *format) {
  if (!file || !format) return fail("null argument");
  *format = file->f.format;
  return J3G_OK;
}

int j3g_nc_nvars(const j3g_ncfile *file, int *nvars) {
  if (!file || !nvars) return fail("null argument");
  *nvars = (int)file->f.vars.size();
  return J3G_OK;
}

int j3g_nc_var_name(const j3g_ncfile *file, int index, int capacity, char *name) {
  if (!file || index < 0 || index >= (int)file->f.vars.size() || !name || capacity < 1)
    return fail("bad variable index");
  const std::string &n = file->f.vars[index].name;
  if ((int)n.size() + 1 > capacity) return fail("name buffer too small");
  std::memcpy(name, n.c_str(), n.size() + 1);
  return J3G_OK;
}

int j3g_nc_var_shape(const j3g_ncfile *file, const char *var, int capacity, int *ndims,
                     long long *shape) {
  if (!file || !var || !ndims) return fail("null argument");
  const Var *v = file->f.find(var);
  if (!v) return fail(std::string("no variable ") + var);
  *ndims = (int)v->shape.size();
  if (capacity < *ndims) return fail("shape buffer too small");
  for (size_t i = 0; i < v->shape.size(); ++i) shape[i] = v->shape[i];
  return J3G_OK;
}

int j3g_nc_read_var(const j3g_ncfile *file, const char *var, long long count, double *values) {
  if (!file || !var) return fail("null argument");
  const Var *v = file->f.find(var);
  if (!v) return fail(std::string("no variable ") + var);
  if (count != (long long)v->values.size())
    return fail(std::string("variable ") + var + " has " + std::to_string(v->values.size()) +
                " values");
  if (count > 0 && !values) return fail("null buffer");
  std::copy(v->values.begin(), v->values.end(), values);
  return J3G_OK;
}

int j3g_nc_dim_len(const j3g_ncfile *file, const char *dim, long long *len) {
  if (!file || !dim || !len) return fail("null argument");
  for (auto &d : file->f.dims)
    if (d.first == dim) {
      *len = d.second;
      return J3G_OK;
    }
  return fail(std::string("no dimension ") + dim);
}

int j3g_nc_text_att(const j3g_ncfile *file, const char *var, const char *att, int capacity,
                    char *value) {
  if (!file || !att || !value || capacity < 1) return fail("null argument");
  const std::map<std::string, std::string> *m = &file->f.text_atts;
  if (var) {
    const Var *v = file->f.find(var);
    if (!v) return fail(std::string("no variable ") + var);
    m = &v->text_atts;
  }
  const auto it = m->find(att);
  if (it == m->end()) return fail(std::string("no text attribute ") + att);
  if ((int)it->second.size() + 1 > capacity) return fail("attribute buffer too small");
  std::memcpy(value, it->second.c_str(), it->second.size() + 1);
  return J3G_OK;
}

int j3g_nc_create(const char *path, j3g_ncwriter **writer) {
  if (!path || !writer) return fail("null argument");
  auto w = std::make_unique<j3g_ncwriter>();
  w->w.path = path;
  *writer = w.release();
  return J3G_OK;
}

int j3g_nc_def_dim(j3g_ncwriter *writer, const char *name, long long len) {
  if (!writer || !name || len < 1 || len > 0x7FFFFFFF) return fail("bad dimension");
  for (auto &d : writer->w.dims)
    if (d.first == name) return fail(std::string("dimension ") + name + " exists");
  writer->w.dims.push_back({name, len});
  return J3G_OK;
}

int j3g_nc_def_var(j3g_ncwriter *writer, const char *name, int type, int ndims,
                   const char *const *dims) {
  if (!writer || !name || ndims < 0 || (ndims > 0 && !dims)) return fail("null argument");
  if (type != J3G_NC_DOUBLE && type != J3G_NC_INT && type != J3G_NC_FLOAT)
    return fail("variables are NC_DOUBLE, NC_FLOAT or NC_INT");
  if (writer->w.find(name)) return fail(std::string("variable ") + name + " exists");
  Writer::WVar v;
  v.name = name;
  v.type = type;
  for (int i = 0; i < ndims; ++i) {
    int id = -1;
    for (size_t k = 0; k < writer->w.dims.size(); ++k)
      if (writer->w.dims[k].first == dims[i]) id = (int)k;
    if (id < 0) return fail(std::string("no dimension ") + dims[i]);
    v.dimids.push_back(id);
  }
  writer->w.vars.push_back(v);
  return J3G_OK;
}

int j3g_nc_put_text_att(j3g_ncwriter *writer, const char *var, const char *name,
                        const char *value) {
  if (!writer || !name || !value) return fail("null argument");
  std::vector<std::pair<std::string, std::string>> *a = &writer->w.gatts;
  if (var) {
    Writer::WVar *v = writer->w.find(var);
    if (!v) return fail(std::string("no variable ") + var);
    a = &v->atts;
  }
  for (auto &x : *a)
    if (x.first == name) {
      x.second = value;
      return J3G_OK;
    }
  a->push_back({name, value});
  return J3G_OK;
}

int j3g_nc_put_var(j3g_ncwriter *writer, const char *var, long long count, const double *values) {
  if (!writer || !var) return fail("null argument");
  Writer::WVar *v = writer->w.find(var);
  if (!v) return fail(std::string("no variable ") + var);
  if (count != writer->w.count(*v))
    return fail(std::string("variable ") + var + " takes " +
                std::to_string(writer->w.count(*v)) + " values");
  if (count > 0 && !values) return fail("null buffer");
  v->values.assign(values, values + count);
  v->put = true;
  return J3G_OK;
}

int j3g_nc_discard_writer(j3g_ncwriter *writer) {
  delete writer;
  return J3G_OK;
}

int j3g_nc_close_writer(j3g_ncwriter *writer) {
  if (!writer) return fail("null argument");
  int rc = J3G_OK;
  try {
    writer->w.write();
  } catch (const std::exception &e) {
    rc = fail(e.what());
  }
  delete writer;
  return rc;
}

}  // extern "C"
