/*
 * Seeded stand-in for std::random_device (test infrastructure only; forced
 * into one golden tool's build by -include, see oracle/Makefile).
 *
 * The reference's SA-1TDVP stage seeds a fresh mt19937 from std::random_device
 * before every group of draws (util/allocation.h:277-278, 308-309;
 * holstein/svd.h:532-534), so no two runs agree.  Compiled with this header,
 * every random_device the reference constructs returns the next value of one
 * mt19937 stream seeded by the environment variable KV_SA_SEED (default 1):
 * the reference's SA stage then repeats run to run, and the oracle, which
 * draws its seeds from the same stream in the same order, can be compared
 * with it.  The reference names the type through `using std::random_device`
 * (util/allocation.h:25), so the stand-in is declared in namespace std.
 */
#ifndef KV_SEEDED_DEVICE_H
#define KV_SEEDED_DEVICE_H
#include <cstdlib>
#include <random>

namespace std {
struct kv_seeded_device {
    unsigned int operator()() {
        static std::mt19937 seeds = [] {
            const char *e = std::getenv("KV_SA_SEED");
            return std::mt19937((std::mt19937::result_type)(e ? std::strtoul(e, nullptr, 10) : 1ul));
        }();
        return (unsigned int)seeds();
    }
};
}  // namespace std

#define random_device kv_seeded_device

#endif
