// h5lite.h -- the small part of the HDF5 file format the dagtm driver needs.
//
// The reference reads its input (T, id, lb) and writes checkpoints and
// outputs through parallel HDF5 (comm/h5comm.c, dagtm/dagtm.cxx:182-431):
// every dataset is created with default properties, i.e. a contiguous
// layout, 2-D matrices row-major and scalars as one-element 1-D datasets,
// all in the root group.  No HDF5 library is available here, so this file
// reads and writes that part of the format:
//   superblock version 0, a root group held in a symbol table (version-1
//   B-tree and local heap), version-1 object headers, datasets of
//   little-endian IEEE float64 / float32 and signed int32 / int64.
// The reader also takes compact and chunked datasets (layout message
// version 3; chunks indexed by a version-1 B-tree), with the deflate (zlib)
// and shuffle filters, as HDF5 tools such as h5repack write them and as the
// reference's sample output data/Oil.out.h5 is stored; the writer writes
// contiguous datasets only.  Every offset read from a file is checked
// against the file's size: a truncated or malformed file gives an error,
// never a read outside the buffer.
// Files written here open with any HDF5 reader; files written by the
// reference (HDF5 1.8 defaults) open here.
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <vector>

namespace h5lite {

struct Dataset {
    std::vector<uint64_t> dims;
    std::vector<double> f64;    // filled for floating-point data (converted)
    std::vector<int64_t> i64;   // filled for integer data
    bool is_int = false;
};

// Read every dataset of the root group (contiguous, compact or chunked).
// Returns false and fills `err` when the file uses a feature outside the
// subset above or is malformed.
bool read_file(const std::string &path, std::map<std::string, Dataset> &out, std::string &err);

class Writer {
  public:
    void add_f64(const std::string &name, const std::vector<uint64_t> &dims, const double *data);
    void add_i32(const std::string &name, const std::vector<uint64_t> &dims, const int32_t *data);
    void add_scalar_f64(const std::string &name, double v) { add_f64(name, {1}, &v); }
    void add_scalar_i32(const std::string &name, int32_t v) { add_i32(name, {1}, &v); }
    bool write(const std::string &path, std::string &err) const;

  private:
    struct Item {
        std::string name;
        std::vector<uint64_t> dims;
        bool is_int;
        std::vector<uint8_t> bytes;
    };
    std::vector<Item> items_;
};

}  // namespace h5lite
