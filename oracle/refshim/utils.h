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
#include <complex>
#include <functional>
#include <map>
#include <numeric>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <sstream>
#include <iostream>
#include <string>
#include <tuple>
#include <utility>
#include <vector>
using namespace std;

/* XLibs helpers used by src/singlepulse/candidate.cpp (their source is not in the reference
 * tree); these are the definitions the GPU path follows.
 * kadane: maximum-sum window, a new maximum needs a strictly larger sum, the running sum
 * restarts after it drops below zero. */
template <typename T> T kadane(const T *a, long int n, long int *start, long int *end)
{
    T best = -INFINITY, cur = 0;
    long int cs = 0;
    *start = 0;
    *end = -1;
    for (long int i = 0; i < n; i++) {
        cur = cur + a[i];
        if (cur > best) {
            best = cur;
            *start = cs;
            *end = i;
        }
        if (cur < 0) {
            cur = 0;
            cs = i + 1;
        }
    }
    return best;
}

/* YMW16 distance (the plot annotation only): not modelled. */
inline double get_dist_ymw16(double, double, double) { return 0.; }

/* get_mean_var: mean and variance of n values, accumulated in double in index order,
 * var = sum(x^2)/n - mean^2. */
template <typename It> void get_mean_var(It begin, long int n, double &mean, double &var)
{
    double s1 = 0., s2 = 0.;
    It it = begin;
    for (long int i = 0; i < n; i++, ++it) {
        const double v = *it;
        s1 += v;
        s2 += v * v;
    }
    mean = s1 / n;
    var = s2 / n - mean * mean;
}
#endif
