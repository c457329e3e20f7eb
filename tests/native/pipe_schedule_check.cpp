// Checks the read schedule the pipelined FP64 Poisson solve relies on
// (PoissonLU::first_read_chunk, used by k64_moments_poisson): for every row k, the forward
// chunk whose staging gathers k's right-hand side must come no later than the first step
// of the sweep that reads x[k], and no gather may touch a row the sweep writes while it
// runs beside it.  The reads are derived here from the factor's band form on their own
// terms: the band's last lane takes up row i + 4 at step i, the first rows enter before
// step 0, and an accumulator lane takes up its row at the step slot_load names; each
// operand is loaded one step ahead of its use (the last step of a chunk loads the next
// chunk's first operands too).  The schedule must give every row exactly its first read.
// Prints a summary and exits non-zero on the first violation.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "poisson_lu.hpp"

int main() {
    const int R = 256;
    int checked = 0;
    for (int n : {5, 17, 64, 100, 255, 256, 257, 1000, 2048, 4096, 8192, 12345, 16384}) {
        vx::PoissonLU lu;
        if (lu.build(n) != 0) {
            std::printf("n=%d: factorisation failed\n", n);
            return 1;
        }
        const vx::PoissonLU::Band Lb = lu.lower_band();
        const std::vector<int> fc = lu.first_read_chunk(Lb, R);
        if (Lb.nslots < 0) {
            if (!fc.empty()) {
                std::printf("n=%d: a schedule for the unpipelined sweep form\n", n);
                return 1;
            }
            continue;
        }
        if ((int)fc.size() != n) {
            std::printf("n=%d: schedule has %zu rows\n", n, fc.size());
            return 1;
        }
        // the chunk during which the sweep first loads the operand of `step`: one step ahead,
        // also across a chunk boundary (the last step of a chunk loads the next chunk's first
        // operands, which its start then loads again)
        auto chunk_of_load = [&](int step) { return step <= 0 ? 0 : (step - 1) / R; };
        std::vector<int> need(n, 1 << 30);
        for (int k = 0; k < std::min(n, 5); k++) need[k] = 0;  // rows 0..3 before step 0, row 4 at step 0
        for (int k = 5; k < n; k++) need[k] = std::min(need[k], chunk_of_load(k - 4));
        for (int s = 0; s < Lb.nslots; s++)
            for (int i = 0; i < n; i++) {
                const int r = Lb.slot_load[(size_t)s * n + i];
                if (r >= 0) need[r] = std::min(need[r], chunk_of_load(i));
            }
        for (int k = 0; k < n; k++) {
            if (fc[k] != need[k]) {  // > : read before it is gathered; < : waits for moments it does not need yet
                std::printf("n=%d: row %d gathered for chunk %d, first read in chunk %d\n", n, k, fc[k], need[k]);
                return 1;
            }
            if (fc[k] < 0 || fc[k] > need[k]) {
                std::printf("n=%d: row %d gathered for chunk %d, read in chunk %d\n", n, k, fc[k], need[k]);
                return 1;
            }
            // the sweep writes x[k] during chunk k / R; the gather of chunk c + 1 runs while
            // chunk c is swept, so it must not be the chunk after the one that writes k
            if (fc[k] > k / R) {
                std::printf("n=%d: row %d gathered for chunk %d after it is written in chunk %d\n", n, k, fc[k],
                            k / R);
                return 1;
            }
        }
        checked++;
    }
    std::printf("pipelined solve schedule: %d sizes consistent\n", checked);
    return 0;
}
