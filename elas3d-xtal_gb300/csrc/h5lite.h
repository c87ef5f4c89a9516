// Minimal HDF5 reader and writer for the solver's input and output files,
// written from the HDF5 file-format specification (version 0/1 superblock,
// version 1 object headers, symbol-table groups with a version-1 B-tree, a
// local heap and symbol-table nodes; contiguous or compact dataset storage).
// That subset is what the HDF5 library writes by default -- the reference's
// MATLAB generator (h5create / h5write / h5writeatt,
// src/microstructure_gen.m:876-889) and its Fortran writer
// (src/elas3dxtal_pcg.f90:2840-2874) both produce files of this form -- so the
// solver reads and writes its HDF5 files without libhdf5, which neither this
// build's hosts nor its GPU hosts provide.
//
// Reader: datasets of the root group by name; fixed-point (1, 2, 4, 8 bytes,
// signed or unsigned) and IEEE floating-point (4, 8 bytes) element types in
// either byte order, converted to int32 / double; object-header continuation
// blocks followed; other messages (attributes, fill values, times) skipped
// except the int32 attribute "dimensions" the MATLAB generator writes.
// Chunked or filtered storage, newer superblocks and dense-link groups are
// reported as unsupported.
//
// Writer: one file with a root group holding 1- or 2-D contiguous datasets of
// int32 or float64 (little endian), each optionally carrying an int32
// attribute, laid out as the HDF5 library lays out such a file.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace h5lite {

enum class Type { I32, F64 };

struct DatasetOut {
  std::string name;
  Type type;
  std::vector<uint64_t> dims;  // HDF5 (C) order, slowest first
  const void* data;            // prod(dims) elements of `type`
  std::string attr_name;       // empty: no attribute
  std::vector<int32_t> attr;   // int32 values of the 1-D attribute
};

// Writes the datasets (names need not be sorted) to path.  Returns 0, or -1 on
// an I/O error.
int write_file(const std::string& path, const std::vector<DatasetOut>& sets);

struct DatasetInfo {
  std::vector<uint64_t> dims;
  int klass = -1;        // 0 fixed-point, 1 floating-point
  int size = 0;          // bytes per element
  bool big_endian = false;
  bool is_signed = true;
  int layout = -1;       // 0 compact, 1 contiguous
  uint64_t addr = 0;     // contiguous: file address of the data (UNDEF: never written)
  uint64_t nbytes = 0;   // bytes of raw data
  std::vector<uint8_t> compact;  // compact: the data
  std::vector<int32_t> dimensions_attr;  // the int32 attribute "dimensions", if present
  uint64_t count() const {
    uint64_t n = 1;
    for (uint64_t d : dims) n *= d;
    return n;
  }
};

class Reader {
 public:
  // Opens path and indexes the root group.  ok() tells whether that worked;
  // error() says why not.
  explicit Reader(const std::string& path);
  bool ok() const { return ok_; }
  bool io_error() const { return io_error_; }  // the file could not be opened or read
  const std::string& error() const { return err_; }
  std::vector<std::string> names() const;
  // Header of dataset `name` (false if absent or not a supported dataset).
  bool info(const std::string& name, DatasetInfo& out);
  // Reads dataset `name` converted to int32 / double; n must equal its element
  // count.  Integer conversion rejects values outside the int32 range.
  bool read_i32(const std::string& name, int32_t* out, uint64_t n);
  bool read_f64(const std::string& name, double* out, uint64_t n);

 private:
  bool fail(const std::string& why);
  bool rd(uint64_t addr, void* dst, uint64_t n);
  uint64_t u(const uint8_t* p, int nbytes) const;
  bool parse_superblock();
  bool walk_btree(uint64_t addr, uint64_t heap_data, int depth);
  bool parse_object_header(uint64_t addr, DatasetInfo& out);
  bool parse_messages(const uint8_t* p, uint64_t len, DatasetInfo& out, std::vector<std::pair<uint64_t, uint64_t>>& cont,
                      bool& have_space, bool& have_type, bool& have_layout);
  bool raw(const DatasetInfo& d, std::vector<uint8_t>& bytes);

  std::vector<uint8_t> file_;
  uint64_t base_ = 0;  // base address (user block size)
  int so_ = 8, sl_ = 8;  // sizes of offsets and lengths
  std::vector<std::pair<std::string, uint64_t>> links_;  // name -> object header address
  bool ok_ = false;
  bool io_error_ = false;
  std::string err_;
};

}  // namespace h5lite
