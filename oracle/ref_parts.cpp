// ref_parts.cpp -- TEST INFRASTRUCTURE.  A C ABI around the two pieces of
// the so3g reference that compile standalone: include/so_linterp.h (the
// asin/atan2 interpolation tables) and src/healpix_bare.c (HEALPix
// ang2ring/ang2nest).  It is compiled from the reference sources where they
// lie (never copied into this repository) by oracle/build.py into
// oracle/_ref/, and is used only to generate and check the golden vectors
// in tests/golden/ that pin the oracle's restatement of those pieces.
#include <cmath>
#include <algorithm>
#include <cstring>
#include "so_linterp.h"
extern "C" {
#include "healpix_bare.h"
}

static asinTable *g_asin = nullptr;
static atan2Table *g_atan2 = nullptr;

static void ensure() {
    if (!g_asin) {
        // TRIG_TABLE_SIZE of src/Projection.cxx:34
        g_asin = new asinTable(1 << 14);
        g_atan2 = new atan2Table(1 << 14);
    }
}

extern "C" {

double ref_asin(double x) { ensure(); return g_asin->get(x); }
double ref_atan2(double y, double x) { ensure(); return g_atan2->get(y, x); }

int ref_tables(double *a, double *b, int n) {
    ensure();
    if (n != g_asin->n) return -1;
    std::memcpy(a, g_asin->vals.data(), sizeof(double) * n);
    std::memcpy(b, g_atan2->vals.data(), sizeof(double) * n);
    return 0;
}

long long ref_ang2ring(long long nside, double theta, double phi) {
    t_ang a = {theta, phi};
    return ang2ring(nside, a);
}

long long ref_ang2nest(long long nside, double theta, double phi) {
    t_ang a = {theta, phi};
    return ang2nest(nside, a);
}

long long ref_nest2ring(long long nside, long long ipix) { return nest2ring(nside, ipix); }
long long ref_ring2nest(long long nside, long long ipix) { return ring2nest(nside, ipix); }

// The sweep of so3g's test_trig (src/so_linterp.cxx:8-36): worst absolute
// discrepancy of the tables against libm over the same grid of inputs.
double ref_trig_worst(int table_size) {
    double worst = 0.;
    double lo = -1., hi = 1., step = .01;
    asinTable asin_lt(table_size);
    for (double x = lo; x < hi; x += step)
        worst = std::max(worst, std::abs(asin_lt.get(x) - asin(x)));
    atan2Table atan2_lt(table_size);
    for (double _x = -3; _x < 3.1; _x += 0.5)
        for (double _y = lo; _y < hi; _y += step)
            worst = std::max(worst, std::abs(atan2_lt.get(_y, _x) - atan2(_y, _x)));
    return worst;
}

}
