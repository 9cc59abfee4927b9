// The reprojection launch rule (isti_launch.cuh) on host: register cap and output row pairs
// per shape class.  Without a device the per-SM limits are the GB300's (65,536 registers,
// 228 KiB of shared memory, 2,048 threads, 32 blocks, 1 KiB reserved per block).
#include "isti_launch.cuh"

#include <cstdio>

int main()
{
    struct Case
    {
        int sw, views, frames, regs, row_pairs;
    };
    // 40 registers with 4+ views except where shared memory already bounds the resident
    // blocks (6 frames: 6 views 6 blocks per SM either way, 4 views 9)
    const Case cases[] = {
        {1, 6, 3, 40, 1}, {1, 6, 1, 40, 3}, {1, 6, 2, 40, 1}, {1, 6, 6, 48, 1}, {1, 4, 6, 48, 1}, {1, 4, 3, 40, 1},
        {1, 4, 1, 40, 2}, {1, 2, 1, 48, 1}, {1, 2, 3, 48, 1}, {1, 2, 6, 48, 1}, {3, 2, 1, 56, 1}, {3, 6, 1, 56, 3},
    };
    int bad = 0;
    for (const Case &c : cases)
    {
        const int rp = isti::rule_row_pairs(c.views, c.frames);
        const int regs = isti::rule_regs(c.sw, c.views, c.frames, rp);
        if (rp != c.row_pairs || regs != c.regs)
        {
            std::printf("window %d, %d views, %d frames: %d registers, %d row pairs; expected %d, %d\n", c.sw, c.views, c.frames, regs, rp,
                        c.regs, c.row_pairs);
            bad++;
        }
    }
    // resident blocks at the GB300 limits: 6 views, 3 frames (20,752 bytes of shared memory)
    const int b40 = isti::resident_blocks(40, 6, isti::reproj_smem<1>(6, 3)), b48 = isti::resident_blocks(48, 6, isti::reproj_smem<1>(6, 3));
    if (b40 != 8 || b48 != 7)
    {
        std::printf("resident blocks %d / %d, expected 8 / 7\n", b40, b48);
        bad++;
    }
    if (bad)
        return 1;
    std::printf("ok %zu cases\n", sizeof(cases) / sizeof(cases[0]));
    return 0;
}
