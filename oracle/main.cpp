/*
 * oracle/main.cpp - entry point of the CPU oracle binary (gsnp_oracle).
 *
 * TEST INFRASTRUCTURE (see oracle/oracle.h).
 */
#include "oracle.h"

int main(int argc, char** argv) { return oracle_main(argc, argv); }
