#pragma once
// Part of the ParlayLib-API stand-in (test infrastructure only).
#include "../psc_parlay_shim.h"
