/* ORACLE / TEST INFRASTRUCTURE ONLY: forced-include prelude that supplies the
 * standard headers the reference's neuron sources use without including. */
#include <cmath>
#include <string>
#include <vector>
#include <functional>
#include <iostream>
#include <numeric>
#include <algorithm>
using std::isnan;
