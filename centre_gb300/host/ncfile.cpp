// ncfile.cpp -- NetCDF classic reader and writer (see ncfile.hpp).
#include "ncfile.hpp"

#include <algorithm>
#include <cstring>

namespace centre_host {
namespace {

constexpr uint32_t kTagDim = 0x0A, kTagVar = 0x0B, kTagAtt = 0x0C;

uint64_t pad4(uint64_t n) { return (4 - n % 4) % 4; }

// big-endian byte string -> native value of size n (1, 2, 4, 8)
void swap_into(const uint8_t *src, uint8_t *dst, size_t n) {
  for (size_t i = 0; i < n; ++i) dst[i] = src[n - 1 - i];
}

bool host_is_little() {
  const uint16_t x = 1;
  return *(const uint8_t *)&x == 1;
}

// Convert count elements of a classic type from big-endian bytes to T.
template <class T>
void decode(int type, const uint8_t *src, uint64_t count, T *dst) {
  const size_t sz = nc_type_size(type);
  const bool le = host_is_little();
  uint8_t tmp[8];
  for (uint64_t i = 0; i < count; ++i) {
    const uint8_t *s = src + i * sz;
    if (le) swap_into(s, tmp, sz);
    else memcpy(tmp, s, sz);
    T v{};
    switch (type) {
      case kNcByte: v = (T)(*(const int8_t *)tmp); break;
      case kNcChar:
      case kNcUByte: v = (T)(*(const uint8_t *)tmp); break;
      case kNcShort: { int16_t a; memcpy(&a, tmp, 2); v = (T)a; break; }
      case kNcUShort: { uint16_t a; memcpy(&a, tmp, 2); v = (T)a; break; }
      case kNcInt: { int32_t a; memcpy(&a, tmp, 4); v = (T)a; break; }
      case kNcUInt: { uint32_t a; memcpy(&a, tmp, 4); v = (T)a; break; }
      case kNcFloat: { float a; memcpy(&a, tmp, 4); v = (T)a; break; }
      case kNcDouble: { double a; memcpy(&a, tmp, 8); v = (T)a; break; }
      case kNcInt64: { int64_t a; memcpy(&a, tmp, 8); v = (T)a; break; }
      case kNcUInt64: { uint64_t a; memcpy(&a, tmp, 8); v = (T)a; break; }
      default: break;
    }
    dst[i] = v;
  }
}

struct Cursor {
  const std::vector<uint8_t> &b;
  size_t o = 0;
  int ver = 1;
  bool ok = true;
  explicit Cursor(const std::vector<uint8_t> &buf) : b(buf) {}
  bool need(uint64_t n) {
    if (!ok || o + n > b.size()) ok = false;
    return ok;
  }
  uint64_t be(int n) {
    if (!need(n)) return 0;
    uint64_t v = 0;
    for (int i = 0; i < n; ++i) v = (v << 8) | b[o + i];
    o += n;
    return v;
  }
  uint32_t u32() { return (uint32_t)be(4); }
  uint64_t nonneg() { return ver == 5 ? be(8) : be(4); }
  uint64_t offset() { return ver == 1 ? be(4) : be(8); }
  std::string name() {
    const uint64_t n = nonneg();
    if (!need(n)) return {};
    std::string s((const char *)&b[o], n);
    o += n + pad4(n);
    return s;
  }
  bool atts(std::vector<NcAtt> &out) {
    const uint32_t tag = u32();
    const uint64_t n = nonneg();
    if (tag == 0 && n == 0) return ok;
    if (tag != kTagAtt) return ok = false;
    for (uint64_t i = 0; i < n && ok; ++i) {
      NcAtt a;
      a.name = name();
      a.type = (int)u32();
      a.count = nonneg();
      const size_t sz = nc_type_size(a.type);
      if (!sz) return ok = false;
      const uint64_t nb = a.count * sz;
      if (!need(nb)) return ok;
      a.raw.resize(nb);
      const bool le = host_is_little();
      for (uint64_t k = 0; k < a.count; ++k) {
        if (le && sz > 1) swap_into(&b[o + k * sz], &a.raw[k * sz], sz);
        else memcpy(&a.raw[k * sz], &b[o + k * sz], sz);
      }
      o += nb + pad4(nb);
      out.push_back(std::move(a));
    }
    return ok;
  }
};

// native -> big-endian append
void put_be(std::vector<uint8_t> &o, uint64_t v, int n) {
  for (int i = n - 1; i >= 0; --i) o.push_back((uint8_t)(v >> (8 * i)));
}

struct HeaderWriter {
  int ver;
  std::vector<uint8_t> h;
  void nonneg(uint64_t v) { put_be(h, v, ver == 5 ? 8 : 4); }
  void u32(uint32_t v) { put_be(h, v, 4); }
  void name(const std::string &s) {
    nonneg(s.size());
    h.insert(h.end(), s.begin(), s.end());
    h.insert(h.end(), pad4(s.size()), 0);
  }
  void atts(const std::vector<NcAtt> &a) {
    if (a.empty()) {
      u32(0);
      nonneg(0);
      return;
    }
    u32(kTagAtt);
    nonneg(a.size());
    const bool le = host_is_little();
    for (const NcAtt &x : a) {
      name(x.name);
      u32((uint32_t)x.type);
      nonneg(x.count);
      const size_t sz = nc_type_size(x.type);
      for (uint64_t k = 0; k < x.count; ++k) {
        uint8_t tmp[8];
        if (le && sz > 1) swap_into(&x.raw[k * sz], tmp, sz);
        else memcpy(tmp, &x.raw[k * sz], sz);
        h.insert(h.end(), tmp, tmp + sz);
      }
      h.insert(h.end(), pad4(x.count * sz), 0);
    }
  }
};

}  // namespace

size_t nc_type_size(int type) {
  switch (type) {
    case kNcByte: case kNcChar: case kNcUByte: return 1;
    case kNcShort: case kNcUShort: return 2;
    case kNcInt: case kNcUInt: case kNcFloat: return 4;
    case kNcDouble: case kNcInt64: case kNcUInt64: return 8;
    default: return 0;
  }
}

NcAtt NcAtt::text(const std::string &name, const std::string &s) {
  NcAtt a;
  a.name = name;
  a.type = kNcChar;
  a.count = s.size();
  a.raw.assign(s.begin(), s.end());
  return a;
}

std::string NcAtt::as_text() const {
  if (type != kNcChar) return {};
  std::string s(raw.begin(), raw.end());
  while (!s.empty() && s.back() == '\0') s.pop_back();
  return s;
}

std::vector<double> NcAtt::as_doubles() const {
  std::vector<double> v(count);
  const size_t sz = nc_type_size(type);
  for (uint64_t i = 0; i < count; ++i) {
    const uint8_t *p = &raw[i * sz];
    switch (type) {
      case kNcByte: v[i] = *(const int8_t *)p; break;
      case kNcChar: case kNcUByte: v[i] = *p; break;
      case kNcShort: { int16_t a; memcpy(&a, p, 2); v[i] = a; break; }
      case kNcUShort: { uint16_t a; memcpy(&a, p, 2); v[i] = a; break; }
      case kNcInt: { int32_t a; memcpy(&a, p, 4); v[i] = a; break; }
      case kNcUInt: { uint32_t a; memcpy(&a, p, 4); v[i] = a; break; }
      case kNcFloat: { float a; memcpy(&a, p, 4); v[i] = a; break; }
      case kNcDouble: { double a; memcpy(&a, p, 8); v[i] = a; break; }
      case kNcInt64: { int64_t a; memcpy(&a, p, 8); v[i] = (double)a; break; }
      case kNcUInt64: { uint64_t a; memcpy(&a, p, 8); v[i] = (double)a; break; }
      default: v[i] = 0; break;
    }
  }
  return v;
}

NcFile::~NcFile() { close(); }

void NcFile::close() {
  if (f_) std::fclose(f_);
  f_ = nullptr;
}

bool NcFile::open(const std::string &path, std::string *err) {
  close();
  path_ = path;
  f_ = std::fopen(path.c_str(), "rb");
  if (!f_) {
    if (err) *err = "cannot open " + path;
    return false;
  }
  std::fseek(f_, 0, SEEK_END);
  file_size_ = (uint64_t)std::ftell(f_);
  std::fseek(f_, 0, SEEK_SET);
  // the header is read incrementally: grow the buffer until it parses
  std::vector<uint8_t> buf;
  size_t want = 1 << 16;
  for (;;) {
    const size_t n = (size_t)std::min<uint64_t>(want, file_size_);
    buf.resize(n);
    std::fseek(f_, 0, SEEK_SET);
    if (std::fread(buf.data(), 1, n, f_) != n) {
      if (err) *err = "short read of " + path;
      return false;
    }
    Cursor c(buf);
    dims.clear();
    atts.clear();
    vars.clear();
    if (n < 4 || memcmp(buf.data(), "CDF", 3) != 0 || !(buf[3] == 1 || buf[3] == 2 || buf[3] == 5)) {
      if (err) *err = path + " is not a NetCDF classic (CDF-1/2/5) file";
      return false;
    }
    c.ver = version = buf[3];
    c.o = 4;
    numrecs = c.nonneg();
    uint32_t tag = c.u32();
    uint64_t nd = c.nonneg();
    if (!(tag == 0 && nd == 0)) {
      if (tag != kTagDim) c.ok = false;
      for (uint64_t i = 0; i < nd && c.ok; ++i) {
        NcDim d;
        d.name = c.name();
        d.len = c.nonneg();
        dims.push_back(d);
      }
    }
    c.atts(atts);
    tag = c.u32();
    const uint64_t nv = c.nonneg();
    if (!(tag == 0 && nv == 0)) {
      if (tag != kTagVar) c.ok = false;
      for (uint64_t i = 0; i < nv && c.ok; ++i) {
        NcVar v;
        v.name = c.name();
        const uint64_t nvd = c.nonneg();
        for (uint64_t k = 0; k < nvd && c.ok; ++k) {
          const uint64_t id = c.nonneg();
          if (id >= dims.size()) c.ok = false;
          v.dimids.push_back((int)id);
        }
        c.atts(v.atts);
        v.type = (int)c.u32();
        v.vsize = c.nonneg();
        v.begin = c.offset();
        if (!nc_type_size(v.type)) c.ok = false;
        vars.push_back(std::move(v));
      }
    }
    if (c.ok) return true;
    if (n >= file_size_ || want > (1u << 30)) {
      if (err) *err = "malformed NetCDF header in " + path;
      return false;
    }
    want *= 4;
  }
}

const NcVar *NcFile::var(const std::string &name) const {
  for (const NcVar &v : vars)
    if (v.name == name) return &v;
  return nullptr;
}

const NcAtt *NcFile::att(const std::string &name) const {
  for (const NcAtt &a : atts)
    if (a.name == name) return &a;
  return nullptr;
}

const NcAtt *NcFile::var_att(const NcVar &v, const std::string &name) const {
  for (const NcAtt &a : v.atts)
    if (a.name == name) return &a;
  return nullptr;
}

int NcFile::dim_id(const std::string &name) const {
  for (size_t i = 0; i < dims.size(); ++i)
    if (dims[i].name == name) return (int)i;
  return -1;
}

uint64_t NcFile::dim_len(int id) const {
  if (id < 0 || id >= (int)dims.size()) return 0;
  return dims[id].len == 0 ? numrecs : dims[id].len;
}

bool NcFile::is_record(const NcVar &v) const {
  return !v.dimids.empty() && dims[v.dimids[0]].len == 0;
}

uint64_t NcFile::record_bytes() const {
  uint64_t n = 0, nrec = 0;
  const NcVar *only = nullptr;
  for (const NcVar &v : vars)
    if (is_record(v)) {
      n += v.vsize;
      ++nrec;
      only = &v;
    }
  if (nrec == 1) {
    // a single record variable is not padded between records
    uint64_t inner = nc_type_size(only->type);
    for (size_t k = 1; k < only->dimids.size(); ++k) inner *= dims[only->dimids[k]].len;
    return inner;
  }
  return n;
}

std::vector<uint64_t> NcFile::shape(const NcVar &v) const {
  std::vector<uint64_t> s;
  for (int d : v.dimids) s.push_back(dim_len(d));
  return s;
}

bool NcFile::read_bytes(uint64_t off, uint64_t n, uint8_t *dst, std::string *err) const {
  if (off + n > file_size_) {
    if (err) *err = "truncated data in " + path_;
    return false;
  }
  if (std::fseek(f_, (long)off, SEEK_SET) != 0 || std::fread(dst, 1, n, f_) != n) {
    if (err) *err = "read error in " + path_;
    return false;
  }
  return true;
}

template <class T>
bool NcFile::read_rows(const NcVar &v, uint64_t rec0, uint64_t nrec, T *dst,
                       std::string *err) const {
  const size_t sz = nc_type_size(v.type);
  uint64_t inner = 1;
  for (size_t k = 1; k < v.dimids.size(); ++k) inner *= dims[v.dimids[k]].len;
  if (v.dimids.empty()) inner = 1;
  const uint64_t row = inner * sz;
  const uint64_t nrows = v.dimids.empty() ? 1 : dim_len(v.dimids[0]);
  if (rec0 + nrec > nrows) {
    if (err) *err = "rows out of range for " + v.name;
    return false;
  }
  if (!is_record(v)) {
    std::vector<uint8_t> buf(row * nrec);
    if (!read_bytes(v.begin + rec0 * row, buf.size(), buf.data(), err)) return false;
    decode(v.type, buf.data(), inner * nrec, dst);
    return true;
  }
  const uint64_t rb = record_bytes();
  // read runs of whole records (bounded chunks) and pick this variable's slab
  const uint64_t per_chunk = std::max<uint64_t>(1, (64ull << 20) / std::max<uint64_t>(rb, 1));
  std::vector<uint8_t> buf;
  for (uint64_t r = 0; r < nrec; r += per_chunk) {
    const uint64_t k = std::min(per_chunk, nrec - r);
    const uint64_t span = (k - 1) * rb + row;
    buf.resize(span);
    if (!read_bytes(v.begin + (rec0 + r) * rb, span, buf.data(), err)) return false;
    for (uint64_t i = 0; i < k; ++i) decode(v.type, buf.data() + i * rb, inner, dst + (r + i) * inner);
  }
  return true;
}

template <class T>
bool NcFile::read_all(const NcVar &v, std::vector<T> &dst, std::string *err) const {
  uint64_t n = 1;
  for (uint64_t s : shape(v)) n *= s;
  dst.resize(n);
  if (n == 0) return true;
  const uint64_t rows = v.dimids.empty() ? 1 : dim_len(v.dimids[0]);
  return read_rows(v, 0, rows, dst.data(), err);
}

#define CENTRE_NC_INST(T)                                                                      \
  template bool NcFile::read_rows<T>(const NcVar &, uint64_t, uint64_t, T *, std::string *) const; \
  template bool NcFile::read_all<T>(const NcVar &, std::vector<T> &, std::string *) const;
CENTRE_NC_INST(float)
CENTRE_NC_INST(double)
CENTRE_NC_INST(uint8_t)
CENTRE_NC_INST(uint32_t)
CENTRE_NC_INST(int64_t)
CENTRE_NC_INST(uint64_t)
#undef CENTRE_NC_INST

bool nc_write(const std::string &path, const NcOut &out, std::string *err) {
  const int ver = out.version;
  int recdim = -1;
  for (size_t i = 0; i < out.dims.size(); ++i)
    if (out.dims[i].len == 0) recdim = (int)i;
  auto is_rec = [&](const NcOut::Var &v) { return !v.dimids.empty() && v.dimids[0] == recdim; };
  std::vector<uint64_t> vsize(out.vars.size()), slab(out.vars.size());
  for (size_t i = 0; i < out.vars.size(); ++i) {
    const NcOut::Var &v = out.vars[i];
    uint64_t n = nc_type_size(v.type);
    for (size_t k = is_rec(v) ? 1 : 0; k < v.dimids.size(); ++k) n *= out.dims[v.dimids[k]].len;
    slab[i] = n;
    vsize[i] = n + pad4(n);
  }
  auto header = [&](const std::vector<uint64_t> &begins) {
    HeaderWriter w{ver, {}};
    w.h = {'C', 'D', 'F', (uint8_t)ver};
    w.nonneg(out.numrecs);
    if (out.dims.empty()) {
      w.u32(0);
      w.nonneg(0);
    } else {
      w.u32(kTagDim);
      w.nonneg(out.dims.size());
      for (const NcDim &d : out.dims) {
        w.name(d.name);
        w.nonneg(d.len);
      }
    }
    w.atts(out.atts);
    if (out.vars.empty()) {
      w.u32(0);
      w.nonneg(0);
    } else {
      w.u32(kTagVar);
      w.nonneg(out.vars.size());
      for (size_t i = 0; i < out.vars.size(); ++i) {
        const NcOut::Var &v = out.vars[i];
        w.name(v.name);
        w.nonneg(v.dimids.size());
        for (int d : v.dimids) w.nonneg((uint64_t)d);
        w.atts(v.atts);
        w.u32((uint32_t)v.type);
        w.nonneg(vsize[i]);
        put_be(w.h, begins[i], ver == 1 ? 4 : 8);
      }
    }
    return w.h;
  };
  const size_t hlen = header(std::vector<uint64_t>(out.vars.size(), 0)).size();
  std::vector<uint64_t> begins(out.vars.size());
  uint64_t o = hlen;
  size_t nrecvars = 0;
  for (size_t i = 0; i < out.vars.size(); ++i)
    if (!is_rec(out.vars[i])) {
      begins[i] = o;
      o += vsize[i];
    }
  for (size_t i = 0; i < out.vars.size(); ++i)
    if (is_rec(out.vars[i])) {
      begins[i] = o;
      o += vsize[i];
      ++nrecvars;
    }
  std::FILE *f = std::fopen(path.c_str(), "wb");
  if (!f) {
    if (err) *err = "cannot create " + path;
    return false;
  }
  const std::vector<uint8_t> h = header(begins);
  bool ok = std::fwrite(h.data(), 1, h.size(), f) == h.size();
  const bool le = host_is_little();
  std::vector<uint8_t> tmp;
  auto emit = [&](const NcOut::Var &v, const uint8_t *src, uint64_t nbytes, uint64_t padded) {
    const size_t sz = nc_type_size(v.type);
    tmp.resize(padded);
    if (le && sz > 1) {
      for (uint64_t k = 0; k < nbytes / sz; ++k) swap_into(src + k * sz, &tmp[k * sz], sz);
    } else if (nbytes) {
      memcpy(tmp.data(), src, nbytes);
    }
    std::fill(tmp.begin() + nbytes, tmp.end(), 0);
    ok = ok && std::fwrite(tmp.data(), 1, padded, f) == padded;
  };
  for (size_t i = 0; i < out.vars.size() && ok; ++i)
    if (!is_rec(out.vars[i])) emit(out.vars[i], (const uint8_t *)out.vars[i].data, slab[i], vsize[i]);
  for (uint64_t r = 0; r < out.numrecs && ok; ++r)
    for (size_t i = 0; i < out.vars.size() && ok; ++i)
      if (is_rec(out.vars[i]))
        emit(out.vars[i], (const uint8_t *)out.vars[i].data + r * slab[i], slab[i],
             nrecvars > 1 ? vsize[i] : slab[i]);
  ok = (std::fclose(f) == 0) && ok;
  if (!ok && err) *err = "write error on " + path;
  return ok;
}

}  // namespace centre_host
