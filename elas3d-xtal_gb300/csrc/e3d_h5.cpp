// HDF5 microstructure input and full-field output of the solver (C ABI,
// include/e3d_micro.h), on the minimal reader / writer of h5lite.cpp.
//
//   e3d_h5_micro_read   ppixel_hdf5 (src/elas3dxtal_pcg.f90:2879-2990): datasets
//                       "pix" (phase per voxel) and "orientation" (Rodrigues
//                       vectors) with the reference's three checks
//   e3d_h5_micro_write  the file the reference's MATLAB generator writes
//                       (src/microstructure_gen.m:876-889)
//   e3d_h5_fullfield_write  fullfield_poly.h5 of stress_fullfield_OpenMP
//                       (src/elas3dxtal_pcg.f90:2840-2874)
#include <cstdint>
#include <string>

#include "e3d_micro.h"
#include "h5lite.h"

void e3d_record_error_text(const char* text);

namespace {

int32_t reject(int32_t code, const std::string& why) {
  e3d_record_error_text(why.c_str());
  return code;
}

}  // namespace

extern "C" int32_t e3d_h5_micro_info(const char* path, int64_t* npix, int64_t* norient, int32_t dims[3]) {
  if (!path || !npix || !norient) return reject(-2, "e3d_h5_micro_info: null argument");
  h5lite::Reader r(path);
  if (!r.ok()) return reject(r.io_error() ? -1 : -2, "e3d_h5_micro_info: " + r.error());
  h5lite::DatasetInfo p, o;
  if (!r.info("pix", p) || !r.info("orientation", o)) return reject(-2, "e3d_h5_micro_info: " + r.error());
  *npix = (int64_t)p.count();
  *norient = (int64_t)o.count();
  if (dims) {
    dims[0] = dims[1] = dims[2] = 0;
    if (p.dimensions_attr.size() == 3)
      for (int i = 0; i < 3; ++i) dims[i] = p.dimensions_attr[i];
  }
  return 0;
}

extern "C" int32_t e3d_h5_micro_read(const char* path, int64_t ns, int32_t ngrains, int32_t* pix, double* rod) {
  if (!path || !pix || ns < 1 || ngrains < 0 || (ngrains > 0 && !rod))
    return reject(-2, "e3d_h5_micro_read: bad argument");
  h5lite::Reader r(path);
  if (!r.ok()) return reject(r.io_error() ? -1 : -2, "e3d_h5_micro_read: " + r.error());
  h5lite::DatasetInfo p, o;
  if (!r.info("pix", p)) return reject(-2, "e3d_h5_micro_read: " + r.error());
  if ((int64_t)p.count() != ns)  // src/elas3dxtal_pcg.f90:2939-2942
    return reject(-3, "e3d_h5_micro_read: HDF5 pix size (" + std::to_string(p.count()) +
                          ") does not match simulation ns (" + std::to_string(ns) + ")");
  if (!r.read_i32("pix", pix, (uint64_t)ns)) return reject(-2, "e3d_h5_micro_read: " + r.error());
  if (!r.info("orientation", o)) return reject(-2, "e3d_h5_micro_read: " + r.error());
  if ((int64_t)o.count() != 3LL * ngrains)  // :2966-2969
    return reject(-3, "e3d_h5_micro_read: HDF5 orientation size (" + std::to_string(o.count()) +
                          ") mismatch with allocated (" + std::to_string(3LL * ngrains) + ")");
  if (ngrains > 0 && !r.read_f64("orientation", rod, 3ULL * ngrains))
    return reject(-2, "e3d_h5_micro_read: " + r.error());
  for (int64_t m = 0; m < ns; ++m)  // :2986-2989
    if (pix[m] < 1 || pix[m] > ngrains + 1) return reject(-4, "e3d_h5_micro_read: phase label in pix out of bounds");
  return 0;
}

extern "C" int32_t e3d_h5_micro_write(const char* path, int32_t nx, int32_t ny, int32_t nz, int32_t ngrains,
                                      const int32_t* pix, const double* rod) {
  if (!path || !pix || nx < 1 || ny < 1 || nz < 1 || ngrains < 0 || (ngrains > 0 && !rod))
    return reject(-2, "e3d_h5_micro_write: bad argument");
  const uint64_t ns = (uint64_t)nx * ny * nz;
  // MATLAB stores an N x 1 column as an HDF5 dataspace of 1 x N (its dimensions
  // reversed), with an int32 attribute "dimensions" beside it
  h5lite::DatasetOut p{"pix", h5lite::Type::I32, {1, ns}, pix, "dimensions", {nx, ny, nz}};
  h5lite::DatasetOut o{"orientation", h5lite::Type::F64, {1, 3ULL * ngrains}, rod, "dimensions", {3 * ngrains, 1}};
  if (h5lite::write_file(path, {p, o}) != 0) return reject(-1, std::string("e3d_h5_micro_write: cannot write ") + path);
  return 0;
}

extern "C" int32_t e3d_h5_fullfield_write(const char* path, int64_t ns, const int32_t* pix, const double* vm,
                                          const double* sigma) {
  if (!path || !pix || !vm || !sigma || ns < 1) return reject(-2, "e3d_h5_fullfield_write: bad argument");
  // the Fortran writer's (ns) and (ns, 6) dataspaces appear reversed in the
  // file: stress_tensor is 6 x ns with the voxel index fastest, i.e. the
  // component-major layout of stress_field(ns, 6)
  h5lite::DatasetOut a{"pix", h5lite::Type::I32, {(uint64_t)ns}, pix, "", {}};
  h5lite::DatasetOut b{"vm", h5lite::Type::F64, {(uint64_t)ns}, vm, "", {}};
  h5lite::DatasetOut c{"stress_tensor", h5lite::Type::F64, {6, (uint64_t)ns}, sigma, "", {}};
  if (h5lite::write_file(path, {a, b, c}) != 0)
    return reject(-1, std::string("e3d_h5_fullfield_write: cannot write ") + path);
  return 0;
}

extern "C" int32_t e3d_h5_dataset_size(const char* path, const char* name, int64_t* count, int32_t* rank,
                                       int64_t dims[8]) {
  if (!path || !name || !count) return reject(-2, "e3d_h5_dataset_size: null argument");
  h5lite::Reader r(path);
  if (!r.ok()) return reject(r.io_error() ? -1 : -2, "e3d_h5_dataset_size: " + r.error());
  h5lite::DatasetInfo d;
  if (!r.info(name, d)) return reject(-2, "e3d_h5_dataset_size: " + r.error());
  *count = (int64_t)d.count();
  if (rank) *rank = (int32_t)d.dims.size();
  if (dims)
    for (size_t i = 0; i < 8; ++i) dims[i] = i < d.dims.size() ? (int64_t)d.dims[i] : 0;
  return 0;
}

extern "C" int32_t e3d_h5_read_i32(const char* path, const char* name, int64_t n, int32_t* out) {
  if (!path || !name || !out || n < 0) return reject(-2, "e3d_h5_read_i32: bad argument");
  h5lite::Reader r(path);
  if (!r.ok()) return reject(r.io_error() ? -1 : -2, "e3d_h5_read_i32: " + r.error());
  if (!r.read_i32(name, out, (uint64_t)n)) return reject(-3, "e3d_h5_read_i32: " + r.error());
  return 0;
}

extern "C" int32_t e3d_h5_read_f64(const char* path, const char* name, int64_t n, double* out) {
  if (!path || !name || !out || n < 0) return reject(-2, "e3d_h5_read_f64: bad argument");
  h5lite::Reader r(path);
  if (!r.ok()) return reject(r.io_error() ? -1 : -2, "e3d_h5_read_f64: " + r.error());
  if (!r.read_f64(name, out, (uint64_t)n)) return reject(-3, "e3d_h5_read_f64: " + r.error());
  return 0;
}
