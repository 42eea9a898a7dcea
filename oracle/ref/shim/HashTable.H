#pragma once
#include "scalar.H"
