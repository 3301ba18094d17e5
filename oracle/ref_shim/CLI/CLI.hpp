// Compile-only stand-in for CLI11, so that the reference's command-line entry point
// compiles inside the oracle harness. TEST INFRASTRUCTURE ONLY: the harness never calls
// the reference's CLI main(), so none of these members do any parsing.
#pragma once

#include <string>

namespace CLI {

struct Validator {};
static const Validator PositiveNumber{};

struct Option {
    Option* check(const Validator&) { return this; }
    Option* required() { return this; }
};

class App {
public:
    explicit App(const std::string& = std::string()) {}
    template <typename T>
    Option* add_option(const std::string&, T&, const std::string& = std::string()) { return &opt_; }
    Option* add_flag(const std::string&, bool&, const std::string& = std::string()) { return &opt_; }
    int parse(int, char**) { return 0; }
private:
    Option opt_;
};

}  // namespace CLI

#define CLI11_PARSE(app, argc, argv) (void)(app).parse((argc), (argv))
