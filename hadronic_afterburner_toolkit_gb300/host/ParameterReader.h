// Parameter store read from "key = value  # comment" files and from
// "key=value" command-line arguments.
//
// Interface and semantics of the reference's ParameterReader
// (src/ParameterReader.{h,cpp}): names are stored with every blank and tab
// removed and lower-cased, the value is the first number of the right-hand
// side, later assignments overwrite earlier ones, getVal(name) fails when
// the key is missing and getVal(name, default) warns and returns the
// default.  Failures throw hbt::ParameterError (the reference prints a
// message and exits; the drop-in's main() does the same on the exception).
#pragma once

#include <stdexcept>
#include <string>
#include <vector>

namespace hbt {
struct ParameterError : std::runtime_error {
    explicit ParameterError(const std::string &m) : std::runtime_error(m) {}
};
}  // namespace hbt

class ParameterReader {
  public:
    ParameterReader() = default;
    ~ParameterReader() = default;

    void phraseOneLine(std::string str, std::string commentSymbol = "#");
    void readFromFile(std::string filename);
    void readFromArguments(long argc, char *argv[], std::string commentSymbol = "#",
                           long start_from = 1);
    bool exist(std::string name) const;
    void setVal(std::string name, double value);
    double getVal(std::string name) const;
    double getVal(std::string name, double defaultValue) const;
    void echo() const;

  private:
    std::vector<std::string> names;
    std::vector<double> values;
    long find_(const std::string &name) const;
};
