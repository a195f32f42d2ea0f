// nlist_impl.cuh -- layout of the azp_nlist workspace object (private).
#pragma once

#include <vector>

#include "celllist.cuh"

struct azp_nlist {
    uint32_t N = 0, ntypes = 0, max_nn = 0, n_builds = 0;
    int tpp = 4;  // threads per particle of the pair driver
    double r_buff = 0.0;
    std::vector<double> r_cut;
    bool have_cuts = false;
    // device
    uint32_t* counts = nullptr;
    uint32_t* nbrs = nullptr;
    azp::ListCut* cuts = nullptr;
    uint4* fixed = nullptr;
    uint32_t* cell_of = nullptr;
    uint32_t* slot = nullptr;
    uint32_t* members = nullptr;
    uint32_t* cell_count = nullptr;
    uint32_t* cell_start = nullptr;
    uint32_t ncell_cap = 0;
    uint32_t* scan_tmp = nullptr;
    uint32_t* flags = nullptr;  // [0] overflow max count
    uint32_t* ex_n = nullptr;
    uint32_t* ex_keys = nullptr;
    uint32_t ex_width = 0;
    // pair-driver workspace: derived type-pair table and r_cut / r_on staging
    double* table = nullptr;   // [ntypes^2][12]
    double* cutbuf = nullptr;  // [2][ntypes^2]
    // adjoint workspace: dual-number type-pair records [ntypes^2][12] x (1 + 5) doubles
    double* adj_table = nullptr;
    // DPD driver workspace: FP32 velocity shadow [N] and per-type-pair constants
    float4* vel_f = nullptr;
    double* dpd_table = nullptr;  // [ntypes^2][8]
};

