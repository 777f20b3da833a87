// Runs the integration guide's C++ sample (extracted verbatim into integration_sample.inc by
// tests/test_gpu_cpp_layer.py) and writes its frames as raw doubles.
//   usage: run_integration_sample <dir> <n> <order> <T_final> <dt> <save_every>
#include "integration_sample.inc"

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>

int main(int argc, char** argv) {
    if (argc < 7) return 2;
    const std::string dir = argv[1];
    try {
        const std::vector<MatrixXd> frames =
            run_vortex(std::atoi(argv[2]), std::atoi(argv[3]), std::atof(argv[4]), std::atof(argv[5]), std::atoi(argv[6]));
        std::ofstream f(dir + "/frames.bin", std::ios::binary);
        for (const MatrixXd& m : frames)
            for (long e = 0; e < m.rows(); ++e)
                for (long k = 0; k < m.cols(); ++k) {
                    const double x = m(e, k);
                    f.write(reinterpret_cast<const char*>(&x), sizeof(x));
                }
        std::ofstream(dir + "/frames.txt") << frames.size() << "\n";
    } catch (const std::exception& ex) {
        std::cerr << "error: " << ex.what() << "\n";
        return 1;
    }
    return 0;
}
