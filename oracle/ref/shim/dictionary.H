// Minimal stand-in for OpenFOAM's dictionary.H (the generated initConsts
// functions take a dictionary argument they do not read).
#pragma once
#include "scalar.H"
namespace Foam { struct dictionary {}; }
