// Stand-in for the two boost::filesystem calls the reference makes.
#pragma once
#include <filesystem>
namespace boost {
namespace filesystem {
using std::filesystem::exists;
using std::filesystem::remove;
}  // namespace filesystem
}  // namespace boost
