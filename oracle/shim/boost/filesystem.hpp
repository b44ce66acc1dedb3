// Boost.Filesystem subset (TEST INFRASTRUCTURE) on top of <filesystem>.
#ifndef DFTG_SHIM_BOOST_FILESYSTEM
#define DFTG_SHIM_BOOST_FILESYSTEM
#include <filesystem>
// Boost's header brings in its fstream wrappers, and with them <fstream>;
// the reference relies on that for std::ifstream.
#include <fstream>
#include <string>
namespace boost {
namespace filesystem {
inline bool exists(const std::string &p) { return std::filesystem::exists(p); }
}  // namespace filesystem
}  // namespace boost
#endif
