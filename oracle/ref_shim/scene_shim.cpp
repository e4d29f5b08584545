// Test infrastructure: host shim around the reference's scene loader (PCISPH/src/scenes.cpp:11-149,
// namespace scene, xraw::Data and load_xraw_host), which build_ref.sh compiles in the same pipe. The
// loader needs only utils::read_file (PCISPH/src/utils/file_io.h); this file supplies it and a C entry
// point for ctypes. Nothing here is used by the library.
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace utils {
inline std::string read_file(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) return {};
    std::ostringstream s;
    s << f.rdbuf();
    return s.str();
}
}  // namespace utils
