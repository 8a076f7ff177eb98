// Boost-subset shim (self-written): everything lives in accumulators.hpp.
#include "../accumulators.hpp"
