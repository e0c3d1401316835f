// Stand-in for src/engine/assets/AssetPath.h: the oracle never reads files,
// so no asset path exists.  Oracle build only.
#pragma once
#include <filesystem>
#include <string>

class AssetPathAbs
{
public:
    explicit AssetPathAbs(const std::string& p) : m_Path(p) {}
    bool Exists() const { return false; }
    const std::filesystem::path& path() const { return m_Path; }
    std::string string() const { return m_Path.string(); }
    operator std::string() const { return m_Path.string(); }
private:
    std::filesystem::path m_Path;
};
