// Binomial checkpointing (Griewank 1992; Griewank & Walther, "Algorithm 799: revolve", 2000):
// where the reverse sweep of the discrete adjoint stores its next checkpoint.  Host code only,
// shared by the adjoint (mol_adjoint.cu) and the CPU tests, which compile it on its own.
#pragma once

#include <algorithm>
#include <cstdint>

namespace mol {

// C(c + r, r), the most steps c checkpoints reverse with r forward repetitions; saturates at 1e18.
inline double binomial_steps(int c, int r) {
    double b = 1.0;
    for (int i = 1; i <= r; ++i) {
        b = b * (c + i) / i;
        if (b > 1e18) return 1e18;
    }
    return b;
}

// Steps to advance before storing the next checkpoint when nn >= 2 steps [l, l + nn) are to be
// reversed from the state u_l (held in its own slot) with `spare` >= 1 further slots.  With
// c = spare + 1 checkpoints (u_l's slot counts: it is reused for the left part) and r the least
// repetition count with C(c + r, r) >= nn, the split min(C(c + r - 1, r - 1), nn - C(c - 1 + r - 1,
// r - 1)) is an optimal one: it attains Griewank's minimum r nn - C(c + r, r - 1) forward steps.
// Any split in [1, nn - 1] gives a correct reverse sweep; the clamp keeps it there.
inline int64_t checkpoint_split(int64_t nn, int spare) {
    const int c = spare + 1;
    int r = 1;
    while (binomial_steps(c, r) < (double)nn) ++r;
    const double left = std::min(binomial_steps(c, r - 1), (double)nn - binomial_steps(c - 1, r - 1));
    return (int64_t)std::max(1.0, std::min(left, (double)(nn - 1)));
}

}  // namespace mol
