#pragma once
#include <CGAL/Exact_predicates_inexact_constructions_kernel.h>
