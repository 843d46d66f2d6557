/*
 * Force-included when compiling the Object-MD reference sources for the CPU
 * oracle (test infrastructure).  Without muParser the reference's
 * ParamHandler (src/omd/param.cpp:194-238) still calls the two-argument
 * conversions as_int(string, parser) / as_double(string, parser) that
 * src/omd/omdtool.cpp only defines under OMD_WITH_MUPARSER.  These forward to
 * the one-argument conversions, which is what the reference does for any
 * value that is not a '{...}' expression.
 */
#ifndef OMDG_ORACLE_NOPARSER_H
#define OMDG_ORACLE_NOPARSER_H
#include <string>
namespace omd {
int as_int(std::string);
double as_double(std::string);
inline int as_int(std::string s, void*) { return as_int(s); }
inline double as_double(std::string s, void*) { return as_double(s); }
}
#endif
