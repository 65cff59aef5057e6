#pragma once
// Forwarding header: every absl/glog symbol the reference CPU path uses lives in one shim.
#include "cp_shim.h"
