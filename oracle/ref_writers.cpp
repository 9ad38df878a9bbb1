/*
 * ref_writers.cpp - the reference's own file writers on the host (TEST
 * INFRASTRUCTURE ONLY: tests/golden/make_golden.py writes their files as
 * golden fixtures, against which tests/ pin the library's writers).
 *
 * The reference code is not in this file: oracle/make_ref.py copies
 * print_file_mini (kernel.cu:3109-3173) into oracle/_ref/ref_pfm.inc and
 * the end-of-run block of main (kernel.cu:4109-4221: the .bin dump, the
 * Tecplot files, the axis line and the run summary) into
 * oracle/_ref/ref_endrun.inc.  This file gives them the Header.h values
 * they read (Nmin, M_inf_, chi_ as runtime variables) and wraps the block of
 * main in a function with the names it uses (host_s, host_u, host_TT,
 * name_all).
 */
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "ref_shim.h"

using namespace std;

int ref_Nmin = 2;                         // Header.h:32
double ref_M_inf = 0.5, ref_chi = 17.0;   // Header.h:76-77
#define Nmin ref_Nmin
#define M_inf_ ref_M_inf
#define chi_ ref_chi
#define kvv(x, y, z) (kv(x) + kv(y) + kv(z))
#define Number1 1.0
#define Number2 0.0
#define Number3 0.0
#define Number4 0.0
#define AllNumber ((Number1) + (Number2) + (Number3) + (Number4))

#include "_ref/ref_pfm.inc"

extern "C" {

// print_file_mini of the state (s, u) (K pairs each) to `path`, with
// every stride-th cell; the neutral arrays it reads (and does not print)
// are zeros, as in the reference's main
void ref_print_file_mini(const double* s, const double* u, int stride, double soltime, const char* path)
{
    ref_Nmin = stride;
    std::vector<double> nn1((size_t)K, 0.0), nn3((size_t)K, 0.0);
    std::vector<double3> nn2((size_t)K, double3{0.0, 0.0, 0.0});
    print_file_mini((double2*)s, (double2*)u, nn1.data(), nn2.data(), nn3.data(), std::string(path), soltime);
}

// the end-of-run files of main: name.bin, name_param_for_texplot.txt (the
// header only), name_param_for_texplot_mini.txt, name_param_y=0.txt and
// name_inform.txt
void ref_end_of_run(const double* s, const double* u, double TT, int stride, double mach_inf, double chi,
                    const char* name)
{
    ref_Nmin = stride;
    ref_M_inf = mach_inf;
    ref_chi = chi;
    double2* host_s = (double2*)s;
    double2* host_u = (double2*)u;
    double host_TT_v = TT;
    double* host_TT = &host_TT_v;
    std::string name_all(name);
#include "_ref/ref_endrun.inc"
}

}  // extern "C"
