// Per-shape algorithm choice (CONV2D_ALGO_AUTO).
#include "wg_plan.h"

namespace wg {

int autotune_pick(const problem_t& pr, const conv2d_options_t& opt, int fallback) {
    (void)pr;
    (void)opt;
    return fallback;
}

}  // namespace wg
