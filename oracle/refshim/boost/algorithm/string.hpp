/*
 * ORACLE shim -- test infrastructure only.
 *
 * Stand-in for the Boost string-algorithm header that the reference's
 * analysis headers include (analyze/statistics.h:8).  Boost is not
 * installed here; the statistics code uses nothing from it, so an empty
 * header lets analyze/statistics.h compile unmodified.
 */
#ifndef ORACLE_SHIM_BOOST_ALGORITHM_STRING_HPP
#define ORACLE_SHIM_BOOST_ALGORITHM_STRING_HPP
#endif
