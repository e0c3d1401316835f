// Stand-in for src/engine/assets/AssetPath.h: paths are used as given (the
// tests pass absolute paths) and Exists() asks the file system, as the
// reference's AssetPathAbs::Exists does for its resolved path.  Oracle build only.
#pragma once
#include <filesystem>
#include <string>

class AssetPathAbs
{
public:
    explicit AssetPathAbs(const std::string& p) : m_Path(p) {}
    bool Exists() const { return std::filesystem::exists(m_Path); }
    const std::filesystem::path& path() const { return m_Path; }
    std::string string() const { return m_Path.string(); }
    operator std::string() const { return m_Path.string(); }
private:
    std::filesystem::path m_Path;
};
