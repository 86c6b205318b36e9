// Throwing definitions for the reference's HDF5IO class so that its CPU
// library links without HDF5.  HDF5 I/O is not on the permute/contract path;
// any call into it from the oracle is a test bug and fails loudly.
#include <stdexcept>
#include <uni10/hdf5io/uni10_hdf5io.h>

namespace uni10 {
static void h5_unavailable() {
  throw std::runtime_error("HDF5 is not available in the oracle build");
}
HDF5IO::HDF5IO(const std::string&) { h5_unavailable(); }
HDF5IO::HDF5IO(const std::string&, const bool) { h5_unavailable(); }
HDF5IO::~HDF5IO() {}
H5::Group HDF5IO::getGroup(const std::string&) { h5_unavailable(); return H5::Group(); }
void HDF5IO::saveNumber(const std::string&, const std::string&, int) { h5_unavailable(); }
void HDF5IO::saveNumber(const std::string&, const std::string&, unsigned long) { h5_unavailable(); }
void HDF5IO::saveNumber(const std::string&, const std::string&, double) { h5_unavailable(); }
void HDF5IO::saveNumber(const std::string&, const std::string&, std::complex<double>) { h5_unavailable(); }
void HDF5IO::saveStdVector(const std::string&, const std::string&, const std::vector<int>&) { h5_unavailable(); }
void HDF5IO::saveStdVector(const std::string&, const std::string&, const std::vector<size_t>&) { h5_unavailable(); }
void HDF5IO::saveStdVector(const std::string&, const std::string&, const std::vector<double>&) { h5_unavailable(); }
void HDF5IO::saveStdVector(const std::string&, const std::string&, const std::vector<std::complex<double> >&) { h5_unavailable(); }
void HDF5IO::saveRawBuffer(const std::string&, const std::string&, const size_t, const int*) { h5_unavailable(); }
void HDF5IO::saveRawBuffer(const std::string&, const std::string&, const size_t, const double*) { h5_unavailable(); }
void HDF5IO::saveRawBuffer(const std::string&, const std::string&, const size_t, const std::complex<double>*) { h5_unavailable(); }
int HDF5IO::loadInt(const std::string&, const std::string&) { h5_unavailable(); return 0; }
size_t HDF5IO::loadUlong(const std::string&, const std::string&) { h5_unavailable(); return 0; }
double HDF5IO::loadReal(const std::string&, const std::string&) { h5_unavailable(); return 0; }
std::complex<double> HDF5IO::loadComplex(const std::string&, const std::string&) { h5_unavailable(); return 0; }
void HDF5IO::loadStdVector(const std::string&, const std::string&, std::vector<int>&) { h5_unavailable(); }
void HDF5IO::loadStdVector(const std::string&, const std::string&, std::vector<size_t>&) { h5_unavailable(); }
void HDF5IO::loadStdVector(const std::string&, const std::string&, std::vector<double>&) { h5_unavailable(); }
void HDF5IO::loadStdVector(const std::string&, const std::string&, std::vector<std::complex<double> >&) { h5_unavailable(); }
void HDF5IO::loadRawBuffer(const std::string&, const std::string&, size_t&, int*&) { h5_unavailable(); }
void HDF5IO::loadRawBuffer(const std::string&, const std::string&, size_t&, double*&) { h5_unavailable(); }
void HDF5IO::loadRawBuffer(const std::string&, const std::string&, size_t&, std::complex<double>*&) { h5_unavailable(); }
void HDF5IO::saveBond(const std::string&, const std::string&, const bondType&) { h5_unavailable(); }
void HDF5IO::saveFlag(const std::string&, const std::string&, const rflag&, const cflag&) { h5_unavailable(); }
void HDF5IO::saveQnum(const std::string&, const std::string&, const int&, const parityType&, const parityFType&) { h5_unavailable(); }
void HDF5IO::loadBond(const std::string&, const std::string&, bondType&) { h5_unavailable(); }
void HDF5IO::loadFlag(const std::string&, const std::string&, rflag&, cflag&) { h5_unavailable(); }
void HDF5IO::loadQnum(const std::string&, const std::string&, int&, parityType&, parityFType&) { h5_unavailable(); }
}  // namespace uni10
