// hbt_afterburner.e - command-line drop-in for the reference executable's
// HBT analysis (src/main.cpp): reads ./parameters.dat plus key=value
// arguments, reads the particle samples under ./results and writes the
// HBT_correlation_function_*.dat files there.
#include <chrono>
#include <iostream>
#include <stdexcept>

#include "Analysis.h"

int main(int argc, char *argv[]) {
    std::cout << "*********************************************************" << std::endl
              << "     HBT correlation functions on the GB300 engine" << std::endl
              << "*********************************************************" << std::endl;
    const auto t0 = std::chrono::steady_clock::now();
    try {
        Analysis analysis("results");
        analysis.UpdateParameterDict("parameters.dat", argc, argv);
        analysis.PerformAnalysis();
    } catch (const hbt::ParameterError &e) {
        std::cout << e.what() << std::endl;
        return 255;
    } catch (const std::exception &e) {
        std::cerr << "error: " << e.what() << std::endl;
        return 1;
    }
    const double s =
        std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::cout << "Program totally finished in " << s << " sec." << std::endl;
    return 0;
}
