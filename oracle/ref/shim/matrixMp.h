// src/MatrixMp.cpp:1 includes "matrixMp.h" while the header on disk is
// src/MatrixMp.h; on a case-sensitive file system this forwarder resolves it.
#pragma once
#include "MatrixMp.h"
