// mdcraft::tools::filesystem (mdcraft/tools/filesystem.h): the standard
// library's filesystem namespace under MDcraft's name.
#pragma once
#include <filesystem>
namespace mdcraft {
namespace tools {
namespace filesystem = std::filesystem;
}  // namespace tools
}  // namespace mdcraft
