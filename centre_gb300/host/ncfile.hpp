// ncfile.hpp -- NetCDF classic files (CDF-1, CDF-2, CDF-5), read and write.
//
// The reference moves every stage's data through libnetcdf: BAT trajectories
// in (src/Netcdf_BAT.cpp:236-330), bin files between the stages
// (src/Netcdf_TrjInt.cpp:542-755, CDF-5) and entropy contributions out
// (src/Netcdf_EntContri.cpp:577-769).  libnetcdf is not a dependency here;
// this is the published classic layout (big-endian header of dimensions,
// attributes and variables, then fixed variables, then records with every
// record variable's slab interleaved per record), which libnetcdf reads and
// writes as NC_CLASSIC_MODEL / NC_64BIT_OFFSET / NC_64BIT_DATA.
#pragma once

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

namespace centre_host {

enum NcType : int {
  kNcByte = 1, kNcChar = 2, kNcShort = 3, kNcInt = 4, kNcFloat = 5, kNcDouble = 6,
  kNcUByte = 7, kNcUShort = 8, kNcUInt = 9, kNcInt64 = 10, kNcUInt64 = 11,
};

size_t nc_type_size(int type);

struct NcDim {
  std::string name;
  uint64_t len = 0;   // 0 = the record (unlimited) dimension
};

// An attribute: values kept in native byte order.
struct NcAtt {
  std::string name;
  int type = kNcChar;
  uint64_t count = 0;
  std::vector<uint8_t> raw;

  static NcAtt text(const std::string &name, const std::string &s);
  template <class T>
  static NcAtt values(const std::string &name, int type, const std::vector<T> &v) {
    NcAtt a;
    a.name = name;
    a.type = type;
    a.count = v.size();
    a.raw.resize(v.size() * sizeof(T));
    if (!v.empty()) std::copy((const uint8_t *)v.data(), (const uint8_t *)v.data() + a.raw.size(),
                              a.raw.begin());
    return a;
  }
  std::string as_text() const;
  // values converted to double (numeric attributes)
  std::vector<double> as_doubles() const;
};

struct NcVar {
  std::string name;
  std::vector<int> dimids;
  std::vector<NcAtt> atts;
  int type = kNcFloat;
  uint64_t vsize = 0;
  uint64_t begin = 0;
};

// Reader: header parsed on open, data read on demand.
class NcFile {
 public:
  NcFile() = default;
  NcFile(const NcFile &) = delete;
  NcFile &operator=(const NcFile &) = delete;
  ~NcFile();

  bool open(const std::string &path, std::string *err);
  void close();

  int version = 0;
  uint64_t numrecs = 0;
  std::vector<NcDim> dims;
  std::vector<NcAtt> atts;
  std::vector<NcVar> vars;

  const NcVar *var(const std::string &name) const;
  const NcAtt *att(const std::string &name) const;
  const NcAtt *var_att(const NcVar &v, const std::string &name) const;
  int dim_id(const std::string &name) const;
  uint64_t dim_len(int id) const;   // the record dimension reports numrecs
  bool is_record(const NcVar &v) const;
  uint64_t record_bytes() const;    // bytes from one record to the next
  std::vector<uint64_t> shape(const NcVar &v) const;

  // Elements [rec0, rec0 + nrec) along the first dimension (records for a
  // record variable, rows otherwise) of a variable, every inner element,
  // converted to T: dst holds nrec * (product of the inner dimensions).
  template <class T>
  bool read_rows(const NcVar &v, uint64_t rec0, uint64_t nrec, T *dst, std::string *err) const;

  // A whole variable.
  template <class T>
  bool read_all(const NcVar &v, std::vector<T> &dst, std::string *err) const;

 private:
  bool read_bytes(uint64_t off, uint64_t n, uint8_t *dst, std::string *err) const;
  std::FILE *f_ = nullptr;
  std::string path_;
  uint64_t file_size_ = 0;
};

// Writer input: dimensions, attributes and variables whose data is a
// contiguous native-order array of the full shape (records first).
struct NcOut {
  int version = 5;
  std::vector<NcDim> dims;
  std::vector<NcAtt> atts;
  struct Var {
    std::string name;
    std::vector<int> dimids;
    std::vector<NcAtt> atts;
    int type = kNcFloat;
    const void *data = nullptr;
  };
  std::vector<Var> vars;
  uint64_t numrecs = 0;
};

bool nc_write(const std::string &path, const NcOut &out, std::string *err);

}  // namespace centre_host
