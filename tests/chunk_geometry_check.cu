// Host-only check of the stage kernels' tile geometry: row chunks across
// block rows (chunk_start, chunk_of_row, chunks_in_block_row in runtime.cuh)
// and tiles across block columns, with the index formulas the stage2 and
// stage3 kernels use for their ledger pieces.  Built and run on the CPU by
// tests/test_oracle_and_abi.py; prints "ok" or the first violated property.
// PLANT_SLOT_MISTAKE replaces the slot formula with a wrong one, to show
// that the check fails.
#include <algorithm>
#include <cstdio>
#include <map>
#include <utility>

#include "../app-binary2d_gb300/csrc/runtime.cuh"

using namespace b2d;

// cols_per_warp: 64 for the paired kernel (stage3), 32 for the TMA-staged one (stage2)
static bool check(int nb, int bs, int tw, int rows, int th, int cols_per_warp)
{
    const int N = nb * bs;
    const int C = rows > 0 ? (N + rows - 1) / rows : N / th;
    const int per_row = std::max(bs / tw, 1);
    const int ncol = std::max(tw / bs, 1);
    const int interior_warps = tw / cols_per_warp, wpc = interior_warps / ncol;
    int most = 0;
    for (int b = 0; b < nb; ++b) most = std::max(most, chunks_in_block_row(b, bs, N, C));
    const int stride = most * per_row;   // tiles_per_block of sync_rundev
    std::map<std::pair<int, int>, int> seen;
    auto fail = [&](const char* what, int ti, int tj) {
        std::printf("nb=%d bs=%d tw=%d rows=%d th=%d: %s at tile (%d, %d)\n", nb, bs, tw, rows, th, what, ti, tj);
        return false;
    };
    if (wpc < 1 || wpc * ncol != interior_warps) return fail("warps do not divide the block columns", 0, 0);
    for (int ti = 0; ti < C; ++ti) {
        const int i0 = chunk_start(ti, N, C), TH = chunk_start(ti + 1, N, C) - i0;
        if (TH < 1 || TH > bs) return fail("chunk height outside [1, bs]", ti, 0);
        if (chunk_of_row(i0, N, C) != ti || chunk_of_row(i0 + TH - 1, N, C) != ti) return fail("chunk_of_row", ti, 0);
        const int rb = std::min(bs - i0 % bs, TH), bl = (i0 + TH - 1) / bs;
        for (int r = 0; r < TH; ++r) {
            const int want = r < rb ? (rb < TH ? bl - 1 : bl) : bl;
            if ((i0 + r) / bs != want) return fail("row outside its piece's block row", ti, 0);
        }
        for (int tj = 0; tj < N / tw; ++tj) {
            const int j0 = tj * tw, bj = j0 / bs, lj0 = j0 % bs;
            const int tib = (ti - chunk_of_row(bl * bs, N, C)) * per_row + lj0 / tw;
            for (int w = 0; w < interior_warps; ++w)
                if ((j0 + cols_per_warp * w) / bs - bj != w / wpc) return fail("warp outside its block column", ti, tj);
            const int npiece = (rb < TH ? 2 : 1) * ncol;
            for (int k = 0; k < npiece; ++k) {
                const int c = k % ncol, first = k >= ncol;
                const int brow = bl - first, bcol = bj + c;
#ifdef PLANT_SLOT_MISTAKE   // without the strips per block: slots of two strips collide
                const int piece = (ti - chunk_of_row(brow * bs, N, C)) + tib % per_row;
#else
                const int piece = (ti - chunk_of_row(brow * bs, N, C)) * per_row + tib % per_row;
#endif
                const int pieces = chunks_in_block_row(brow, bs, N, C) * per_row;
                if (brow < 0 || bcol >= nb) return fail("piece outside the mesh", ti, tj);
                if (piece < 0 || piece >= pieces || pieces > stride) return fail("piece slot out of range", ti, tj);
                if (seen.count({brow * nb + bcol, piece})) return fail("piece slot written twice", ti, tj);
                seen[{brow * nb + bcol, piece}] = pieces;
            }
        }
    }
    for (int b = 0; b < nb; ++b)
        for (int c = 0; c < nb; ++c) {
            int n = 0;
            for (auto& kv : seen) n += kv.first.first == b * nb + c;
            if (n != chunks_in_block_row(b, bs, N, C) * per_row) return fail("block arrivals differ from its count", b, c);
        }
    return true;
}

int main()
{
    struct Case { int nb, bs, tw, rows, th, cpw; };
    const Case cases[] = {
        // paired kernel: row chunks, 128/256/512-column tiles over blocks
        {3, 64, 64, 40, 32, 64}, {3, 64, 64, 20, 32, 64}, {2, 128, 128, 100, 32, 64}, {2, 128, 64, 8, 32, 64},
        {2, 128, 256, 100, 32, 64}, {2, 128, 256, 0, 32, 64}, {4, 64, 128, 50, 32, 64}, {4, 128, 512, 100, 32, 64},
        {8, 64, 512, 40, 32, 64}, {16, 128, 512, 54, 64, 64}, {16, 128, 256, 54, 64, 64}, {16, 128, 128, 54, 64, 64},
        {17, 128, 128, 9, 64, 64}, {64, 128, 256, 125, 64, 64},
        // TMA-staged kernel: one column per thread
        {4, 32, 32, 12, 8, 32}, {4, 32, 32, 20, 16, 32}, {3, 64, 32, 20, 16, 32}, {3, 64, 64, 40, 32, 32},
        {32, 128, 128, 98, 64, 32}, {32, 128, 64, 58, 64, 32}, {5, 64, 64, 0, 16, 32},
    };
    for (const Case& c : cases)
        if (!check(c.nb, c.bs, c.tw, c.rows, c.th, c.cpw)) return 1;
    std::printf("ok\n");
    return 0;
}
