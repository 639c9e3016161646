/*
 * utils.h -- stand-in for the XLibs header of the same name, providing only what
 * src/singlepulse/boxcar.cpp and cluster.cpp of the reference need in order to compile in
 * place for the parity harness (standard headers and the std namespace).
 * Test infrastructure only.
 */
#ifndef TXREF_UTILS_H
#define TXREF_UTILS_H
#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <tuple>
#include <utility>
#include <vector>
using namespace std;
#endif
