// Minimal stand-in for OpenFOAM's scalar.H so the reference's generated
// ionic-model headers compile outside OpenFOAM (oracle pinning only).
#pragma once
#include <cmath>
#include <string>
#include <vector>
#include <utility>
#include <initializer_list>
namespace Foam {
typedef double scalar;
typedef int label;
typedef std::string word;
struct wordList : std::vector<std::string> {
    wordList() {}
    wordList(std::initializer_list<std::string> l) : std::vector<std::string>(l) {}
};
template <class T> struct HashTable : std::vector<std::pair<std::string, T>> {
    HashTable(std::initializer_list<std::pair<std::string, T>> l)
        : std::vector<std::pair<std::string, T>>(l) {}
};
using std::exp; using std::log; using std::pow; using std::sqrt; using std::tanh;
using std::fabs; using std::floor;
}
using std::exp; using std::log; using std::pow; using std::sqrt; using std::tanh;
