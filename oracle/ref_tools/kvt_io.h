/*
 * Small helpers shared by the reference-side golden-vector tools.
 *
 * Test infrastructure only: these tools are compiled against the reference
 * Kylin-V headers in place (holstein/*.h) and write golden tensors that the
 * test-suite compares the GPU library and the CPU restatement against.
 *
 * KVT tensor file (little-endian):
 *   int32 magic 0x3154564B ("KVT1"), int32 rank, int32 dirs[rank], int32 nblocks,
 *   then per block: int32 shape[rank], int32 qn[rank], complex128 data[prod(shape)]
 *   (row-major, the same element order as the reference's Block<Rank>,
 *   holstein/block.h:154-161).
 */
#pragma once
#include <cstdio>
#include <cstdint>
#include <string>
#include <vector>

namespace kvt {

static const int32_t kMagic = 0x3154564B;

template <class TensorT, int Rank>
inline void write_tensor(const std::string &path, const TensorT &t) {
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) { std::perror(path.c_str()); std::exit(2); }
    int32_t hdr[2] = {kMagic, Rank};
    std::fwrite(hdr, sizeof(int32_t), 2, f);
    int32_t dirs[Rank];
    for (int i = 0; i < Rank; ++i) dirs[i] = t.dirs()[i];
    std::fwrite(dirs, sizeof(int32_t), Rank, f);
    int32_t nb = t.num_blocks();
    std::fwrite(&nb, sizeof(int32_t), 1, f);
    for (int b = 0; b < nb; ++b) {
        const auto &blk = t.at(b);
        int32_t sh[Rank], qn[Rank];
        for (int i = 0; i < Rank; ++i) { sh[i] = blk.shape()[i]; qn[i] = blk.qn()[i]; }
        std::fwrite(sh, sizeof(int32_t), Rank, f);
        std::fwrite(qn, sizeof(int32_t), Rank, f);
        std::fwrite(blk.cptr(), 16, blk.size(), f);
    }
    std::fclose(f);
}

inline void write_doubles(const std::string &path, const std::vector<double> &v) {
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) { std::perror(path.c_str()); std::exit(2); }
    std::fwrite(v.data(), sizeof(double), v.size(), f);
    std::fclose(f);
}

}  // namespace kvt
