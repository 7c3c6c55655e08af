// Calls simulation::full_dynamics through include/magpy_simulation.hpp, the
// reference's C++ signature (include/simulation.hpp:74-94) over the C-ABI.
//
//   test_simulation_adapter          argument checks only (no GPU needed):
//                                    mismatched inputs, an unknown field
//                                    option and max_samples = 0 throw
//                                    std::invalid_argument before any device work
//   test_simulation_adapter run      a 3-particle run with a sine field,
//                                    printed as "i s mx my mz field time"
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include "magpy_simulation.hpp"

static int expect_invalid(const char *what, void (*f)())
{
    try {
        f();
    } catch (const std::invalid_argument &) {
        return 0;
    } catch (...) {
        std::fprintf(stderr, "%s: wrong exception type\n", what);
        return 1;
    }
    std::fprintf(stderr, "%s: no exception\n", what);
    return 1;
}

static const std::vector<d3> AX{{0, 0, 1}, {0, 1, 0}, {1, 0, 0}};
static const std::vector<d3> LOC{{0, 0, 0}, {2e-8, 0, 0}, {0, 2.1e-8, 0}};

int main(int argc, char **argv)
{
    if (argc > 1 && std::strcmp(argv[1], "run") == 0) {
        auto res = simulation::full_dynamics({7e-9, 6e-9, 6.5e-9}, {2e4, 2.2e4, 1.9e4}, AX, AX, LOC,
                                             4e5, 0.1, 300.0, false, true, false, 1e-9, 1e-13,
                                             2e-11, 11, 4321, field::SINE, 1e4, 3e9);
        for (size_t i = 0; i < res.size(); i++)
            for (size_t s = 0; s < res[i].N; s++)
                std::printf("%zu %zu %.17g %.17g %.17g %.17g %.17g\n", i, s, res[i].mx[s],
                            res[i].my[s], res[i].mz[s], res[i].field[s], res[i].time[s]);
        return simulation::last_status() == 0 ? 0 : 2;
    }
    int bad = 0;
    bad += expect_invalid("mismatched inputs", [] {
        simulation::full_dynamics({7e-9, 6e-9}, {2e4}, AX, AX, LOC, 4e5, 0.1, 300.0, false, true,
                                  false, 1e-9, 1e-13, 2e-11, 11, 1);
    });
    bad += expect_invalid("unknown field option", [] {
        simulation::full_dynamics({7e-9}, {2e4}, {AX[0]}, {AX[0]}, {LOC[0]}, 4e5, 0.1, 300.0,
                                  false, true, false, 1e-9, 1e-13, 2e-11, 11, 1,
                                  (field::options)7);
    });
    bad += expect_invalid("max_samples = 0", [] {
        simulation::full_dynamics({7e-9}, {2e4}, {AX[0]}, {AX[0]}, {LOC[0]}, 4e5, 0.1, 300.0,
                                  false, true, false, 1e-9, 1e-13, 2e-11, 0, 1);
    });
    if (bad == 0) std::printf("checks ok\n");
    return bad;
}
