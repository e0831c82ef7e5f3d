// Driver of the HBT analysis (the HBT part of the reference's Analysis
// class, src/Analysis.{h,cpp}: parameter dictionary, RNG seeding and the
// buffer loop of Analysis::HBTAnalysis, src/Analysis.cpp:817-835).  The
// flow, balance-function and yield analyses are not part of this build and
// are skipped with a warning.
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
    ParameterReader &parameters() { return paraRdr_; }

  private:
    const std::string path_;
    ParameterReader paraRdr_;
    std::shared_ptr<RandomUtil::Random> ran_gen_ptr_;
    std::shared_ptr<particleSamples> particle_list_;
    void setRapidityShiftFromFile();
};
