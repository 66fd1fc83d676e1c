// ORACLE — TEST INFRASTRUCTURE ONLY. Part of the scalar VecCore stand-in (see VecCore).
#include "VecCore"
