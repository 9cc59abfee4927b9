// isti::pack_shadow_entries (include/isti_renderer.hpp) on images read from a file:
// usage: shadow_pack_hpp <in: n_pixels u32, info RGBA, A RGBA, B RGB> <out: entries>
#include "isti_renderer.hpp"

#include <cstdio>
#include <vector>

int main(int argc, char **argv)
{
    if (argc != 3)
        return 2;
    FILE *f = std::fopen(argv[1], "rb");
    if (!f)
        return 3;
    uint32_t n = 0;
    if (std::fread(&n, 4, 1, f) != 1)
        return 4;
    std::vector<uint8_t> info(4 * (size_t)n), a(4 * (size_t)n), b(3 * (size_t)n);
    if (std::fread(info.data(), 1, info.size(), f) != info.size() || std::fread(a.data(), 1, a.size(), f) != a.size() ||
        std::fread(b.data(), 1, b.size(), f) != b.size())
        return 5;
    std::fclose(f);
    const std::vector<uint8_t> e = isti::pack_shadow_entries(info.data(), 4, a.data(), 4, b.data(), 3, n);
    FILE *o = std::fopen(argv[2], "wb");
    if (!o || std::fwrite(e.data(), 1, e.size(), o) != e.size())
        return 6;
    std::fclose(o);
    bool threw = false;
    try
    {
        isti::pack_shadow_entries(info.data(), 2, a.data(), 4, b.data(), 3, n);
    }
    catch (const isti::Error &)
    {
        threw = true;
    }
    std::printf("%s %zu\n", threw ? "ok" : "no-throw", e.size() / ISTI_SHADOW_ENTRY_BYTES);
    return threw ? 0 : 7;
}
