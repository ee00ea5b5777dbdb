// qdg_schedule.h -- FFT schedules (radix order, lines per batch) per line
// length and precision, from the autotuner's table (qdg_schedule.cpp).
#pragma once

namespace qdg {

// Radix plan of one line length: N = prod radix[i], radices in {16, 8, 4, 2, 3, 5}
// or (any_radix) other primes, each a direct DFT stage of O(p^2) work per item.
struct RadixPlan {
  int n;
  int nstages;
  int radix[16];
};

enum ScheduleContext { SCHED_PLAN = 0, SCHED_ENSEMBLE = 1 };

// Largest radices first (16, 8, 4, 2, then 3s and 5s); false unless n = 2^a 3^b 5^c.
bool greedy_radix(int n, RadixPlan &rp);
// Greedy for the 2^a 3^b 5^c part, then every other prime factor ascending;
// false only for n < 1.
bool any_radix(int n, RadixPlan &rp);
// True when a stage has a radix outside {16, 8, 4, 2, 3, 5}.
bool generic_radix(const RadixPlan &rp);
// The tuned order for (context, n, precision), else the greedy one.
bool schedule_radix(int context, int n, int precision, RadixPlan &rp);
// Lines per batch of the step kernel for this line length (0: automatic).
int schedule_lines(int context, int n, int precision);

}  // namespace qdg
