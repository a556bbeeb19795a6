// HDF5 output files of the reference's schema, written without the HDF5
// library (none is linked): the observables time series
// (TDSEZManager::WriteHDF5, src/manager.cpp:51-201) and flat files of
// float64 datasets with float64 attributes on the root group (the t-SURFF
// spectra, src/tsurff.cpp:1018-1057).
//
// The file is the library's classic layout, which every HDF5 reader since
// 1.0 opens: a version-0 superblock, one root group indexed by a version-1
// B-tree with one symbol-table node and a local heap of names, version-1
// object headers, contiguous little-endian IEEE float64 data.
#pragma once

#include <array>
#include <cstdint>
#include <string>
#include <vector>

namespace tdz {

// A float64 dataset or attribute: name, shape (slowest axis first; empty for
// a scalar) and row-major values.
struct H5Array {
    std::string name;
    std::vector<uint64_t> dims;
    const double *data = nullptr;
};

// Writes `path` (parent directories created) holding `datasets` in the root
// group and `attrs` on it. The file is written to path + ".part" and renamed,
// so a reader never sees a partial file. Dataset names are unique, non-empty,
// without '/' or '.', and every dataset has rank 1..8 with no zero extent.
void h5_write_file(const std::string &path, const std::vector<H5Array> &datasets,
                   const std::vector<H5Array> &attrs);

// The observables file of a propagation: five float64 datasets with one row
// per recorded step, rows buffered on the host and the file rewritten when
// `flush_rows` rows are pending, on flush() and on close. Widths by
// dimension (src/manager.cpp:188-192, 395-397):
//   dipoles          1 + 3 dim   t, E_a, D_a, A_a
//   populations      1 + n_bound t, P_0 .. P_{n-1}
//   energies         7           t, Kin, Pot, Int, Tot, InvMass, Norm
//   currents         11 (15 in 3D)
//   autocorrelation  3           t, Re C, Im C
// Column 0 of every dataset is the time of the row; quantities the caller
// does not supply are zero, as for quantities disabled in the reference.
class ObsFile {
  public:
    static constexpr int kSets = 5;
    static const char *const kNames[kSets];

    ObsFile(const std::string &path, int dim, int n_bound, long long flush_rows);
    int columns(int set) const { return cols_[set]; }
    long long rows() const { return nrows_; }
    long long written() const { return written_; }
    // rows[s] holds columns(s) - 1 values (the row after its time), or is
    // null (zeros); rows itself may be null.
    void record(double t, const double *const *rows);
    void flush();

  private:
    std::string path_;
    std::array<int, kSets> cols_{};
    std::array<std::vector<double>, kSets> data_;
    long long nrows_ = 0, written_ = 0, flush_rows_;
};

}  // namespace tdz
