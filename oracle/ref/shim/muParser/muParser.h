/*
 * Test infrastructure (the CPU oracle build only).  muParser is a third-party
 * library that the reference does not vendor.  src/omd/fdtd.cpp defines its
 * expression variables and functions on a global mu::Parser and evaluates an
 * expression only for '{...}' values; this stand-in accepts those calls and
 * evaluates a plain number, and throws (as muParser does on a syntax error)
 * for anything else, so that the oracle build covers constant assignments.
 */
#ifndef OMDG_ORACLE_MUPARSER_STANDIN_H
#define OMDG_ORACLE_MUPARSER_STANDIN_H
#include <cstdlib>
#include <string>

namespace mu {

class ParserError {
    std::string msg_;

public:
    explicit ParserError(const std::string& m) : msg_(m) {}
    const std::string& GetMsg() const { return msg_; }
};

class Parser {
    std::string expr_;

public:
    typedef ParserError exception_type;
    void DefineFun(const char*, double (*)(double, double)) {}
    void DefineConst(const char*, double) {}
    void DefineVar(const char*, double*) {}
    void SetExpr(const std::string& e) { expr_ = e; }
    double Eval() const {
        const char* s = expr_.c_str();
        char* end = 0;
        double v = std::strtod(s, &end);
        while (end && (*end == ' ' || *end == '\t')) end++;
        if (end == s || !end || *end) throw ParserError("expression needs muParser: " + expr_);
        return v;
    }
};

}  // namespace mu
#endif
