/* Minimal stand-in for the HDF5 C++ header, used only to compile the
 * reference library's CPU path as a test oracle in an image without HDF5.
 * Only the class names that the reference's hdf5io header mentions exist
 * here; every HDF5IO method is defined in h5io_stub.cpp to throw. */
#ifndef TRIM_ORACLE_H5CPP_STUB_H
#define TRIM_ORACLE_H5CPP_STUB_H
namespace H5 {
class H5File {
 public:
  H5File() {}
  virtual ~H5File() {}
};
class Group {};
class CompType {};
class EnumType {};
}  // namespace H5
#endif
