// argparse stand-in for the oracle's reference builds: the declarations the
// reference's Arguments wrapper (include/argparse/arguments.hpp) compiles
// against.  Nothing is parsed: every option keeps the value the program
// stored before parsing, so reference programs run with their defaults.
#pragma once
#include <deque>
#include <ostream>
#include <string>

namespace argparse {
class Argument {
 public:
  template <class... A>
  Argument& help(A&&...) { return *this; }
  template <class T>
  Argument& default_value(T&&) { return *this; }
  template <class T>
  Argument& implicit_value(T&&) { return *this; }
  template <class T>
  Argument& store_into(T&) { return *this; }
  template <char Shape, class T>
  Argument& scan() { return *this; }
  Argument& required() { return *this; }
  template <class F>
  Argument& action(F&&) { return *this; }
  template <class... V>
  Argument& choices(V&&...) { return *this; }
};

class ArgumentParser {
 public:
  explicit ArgumentParser(std::string = "") {}
  template <class... N>
  Argument& add_argument(N&&...) {
    args_.emplace_back();
    return args_.back();
  }
  void parse_args(int, char**) {}
  friend std::ostream& operator<<(std::ostream& o, const ArgumentParser&) { return o; }

 private:
  std::deque<Argument> args_;
};
}  // namespace argparse
