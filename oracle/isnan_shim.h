/* Force-included into the reference's MathUtil.cc only: that file calls an
 * unqualified isnan(), which modern libstdc++ no longer puts in the global
 * namespace.  No arithmetic effect. */
#include <cmath>
using std::isnan;
