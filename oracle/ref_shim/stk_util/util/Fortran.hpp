#pragma once
#define SIERRA_FORTRAN(x) x##_
