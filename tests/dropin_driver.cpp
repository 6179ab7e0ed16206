// Exercises the drop-in C++ layer (include/holstein/) the way a reference
// driver does: load an MPS and an MPO in the reference's binary formats, build
// Holstein::TDVP, run total_start on a stage string.  Usage:
//   dropin_driver <mps file> <mpo file> <stage "[nK,n2,0,n1]"> <maxD> <tolSVD>
#include "holstein/tdvp.h"

using namespace KylinVib;

int main(int argc, char **argv) {
    if (argc < 6) return 2;
    ifstream ifs(argv[1]), ifo(argv[2]);
    Holstein::State mps = Holstein::State::load(ifs);
    Holstein::Operator mpo = Holstein::Operator::load(ifo);
    array<INT, 4> stage = Holstein::parse_stage(argv[3]);
    Holstein::TDVP drive(mps, mpo, stod(argv[5]), 1e-8, (INT)stol(argv[4]), 11, 0.05);
    drive.total_start(stage);
    return 0;
}
