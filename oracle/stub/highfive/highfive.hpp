// TEST INFRASTRUCTURE ONLY: a project-written no-op stand-in for the HighFive API that the
// reference's phantom generators use in phantom_base::save() (libhdf5 is not installed here).
// The oracle never saves; it reads the generated mask and field from memory.
#pragma once
#include <string>
#include <vector>

namespace HighFive {
struct DataSpace {
    template <typename T>
    explicit DataSpace(const T &) {}
};
struct DataSet {
    template <typename T>
    void write_raw(const T *) {}
};
struct File {
    enum { Truncate = 0 };
    File(const std::string &, int) {}
    template <typename T>
    DataSet createDataSet(const std::string &, const DataSpace &) { return DataSet(); }
};
}  // namespace HighFive
