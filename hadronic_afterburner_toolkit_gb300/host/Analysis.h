// Driver of the HBT and balance-function analyses (those parts of the
// reference's Analysis class, src/Analysis.{h,cpp}: parameter dictionary,
// RNG seeding and the buffer loops of Analysis::HBTAnalysis and
// Analysis::BalanceFunctionAnalysis, src/Analysis.cpp:817-874).  The flow
// and yield analyses are not part of this library and are skipped with a
// warning.
#pragma once

#include <memory>
#include <string>

#include "ParameterReader.h"
#include "Random.h"
#include "particleSamples.h"

class Analysis {
  public:
    explicit Analysis(std::string path);
    void UpdateParameterDict(std::string param_filename);
    void UpdateParameterDict(std::string param_filename, int argc, char *argv[]);
    void InitializeAnalysis();
    void PerformAnalysis();
    void HBTAnalysis();
    void BalanceFunctionAnalysis();
    ParameterReader &parameters() { return paraRdr_; }

  private:
    const std::string path_;
    ParameterReader paraRdr_;
    std::shared_ptr<RandomUtil::Random> ran_gen_ptr_;
    std::shared_ptr<particleSamples> particle_list_;
    void setRapidityShiftFromFile();
};
