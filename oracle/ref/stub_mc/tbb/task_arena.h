#pragma once
#include "tbb_serial.h"
