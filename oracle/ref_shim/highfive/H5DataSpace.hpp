#pragma once
#include <highfive/H5File.hpp>
