#include "ParameterReader.h"

#include <cctype>
#include <fstream>
#include <iostream>
#include <sstream>

namespace {

// Every blank and tab is dropped (the reference's trim(), src/arsenal.cpp).
std::string squeeze(const std::string &s) {
    std::string out;
    out.reserve(s.size());
    for (char ch : s)
        if (ch != ' ' && ch != '\t') out.push_back(ch);
    return out;
}

std::string lower(std::string s) {
    for (char &ch : s) ch = static_cast<char>(std::tolower(static_cast<unsigned char>(ch)));
    return s;
}

// First number of the string (the reference's stringToDouble).
double first_number(const std::string &s) {
    std::stringstream ss(s + " ");
    double v = 0.0;
    ss >> v;
    return v;
}

}  // namespace

long ParameterReader::find_(const std::string &name) const {
    const std::string key = lower(squeeze(name));
    for (size_t k = 0; k < names.size(); k++)
        if (names[k] == key) return static_cast<long>(k);
    return -1;
}

void ParameterReader::phraseOneLine(std::string str, std::string commentSymbol) {
    if (squeeze(str).empty()) return;
    const std::string eq = str.substr(0, str.find(commentSymbol));
    if (squeeze(eq).empty()) return;
    const size_t at = eq.find('=');
    if (at == std::string::npos)
        throw hbt::ParameterError(
            "ParameterReader::phraseEquationWithoutComments error:\"=\" symbol not found in "
            "equation assignment " + eq);
    setVal(eq.substr(0, at), first_number(squeeze(eq.substr(at + 1))));
}

void ParameterReader::readFromFile(std::string filename) {
    std::ifstream in(filename.c_str());
    if (!in)
        throw hbt::ParameterError("ParameterReader::readFromFile error: file " + filename +
                                  " does not exist.");
    std::string line;
    while (std::getline(in, line)) phraseOneLine(line);
}

void ParameterReader::readFromArguments(long argc, char *argv[], std::string commentSymbol,
                                        long start_from) {
    for (long k = start_from; k < argc; k++) phraseOneLine(argv[k], commentSymbol);
}

bool ParameterReader::exist(std::string name) const { return find_(name) != -1; }

void ParameterReader::setVal(std::string name, double value) {
    const long k = find_(name);
    if (k == -1) {
        names.push_back(lower(squeeze(name)));
        values.push_back(value);
    } else {
        values[k] = value;
    }
}

double ParameterReader::getVal(std::string name) const {
    const long k = find_(name);
    if (k == -1)
        throw hbt::ParameterError("ParameterReader::getVal error: parameter with name " + name +
                                  " not found.");
    return values[k];
}

double ParameterReader::getVal(std::string name, double defaultValue) const {
    const long k = find_(name);
    if (k != -1) return values[k];
    std::cout << "ParameterReader::getVal error: parameter with name " << name
              << " not found." << std::endl;
    std::cout << "using defaultValue: " << defaultValue << std::endl;
    return defaultValue;
}

void ParameterReader::echo() const {
    if (names.empty()) return;
    for (size_t k = 0; k < names.size(); k++) std::cout << names[k] << "=" << values[k] << "  ";
    std::cout << std::endl;
}
