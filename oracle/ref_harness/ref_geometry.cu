// Geometry pin: drives the reference's own host-side node classification
// (sakthi-lbm/MRLBM_3D_CUDA, shipped cylinder case, and the same case with Z_PERIODIC 0 for
// the BCSOLID nodes of cases/cylinder/nodeClass.cuh:254-287) and dumps its result, so the
// oracle's and the product's restatements can be checked against it.  Test infrastructure only.
//
// Compiled by oracle/build_ref.py from the reference sources where they lie
// (-I <reference>/MRLBM_3D/src); nothing here runs on a GPU: only inline host functions of
//   solver/initializeLBM.cuh:58-80 (initialize_nodeType -> boundary_definitions),
//   cases/cylinder/nodeClass.cuh:289-324 (initialize_cylinder_nodeType_triangular / _staircase),
//   cases/cylinder/cylinder_helpers.cuh:10-299 (lists, indices, normals, masks)
// are called, on malloc'd arrays in place of the cudaMallocHost ones of
// cylinder_kernels.cuh:406-465.
#include <cstdio>
#include <cstdlib>
#include <filesystem>
#include <string>
#include <unistd.h>

#include "solver/initializeLBM.cuh"

static void dump(const std::string &dir, const char *name, const void *p, size_t bytes) {
    const std::string path = dir + "/" + name;
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) {
        fprintf(stderr, "cannot write %s\n", path.c_str());
        exit(2);
    }
    fwrite(p, 1, bytes, f);
    fclose(f);
}

int main(int argc, char **argv) {
    if (argc < 2) {
        fprintf(stderr, "usage: ref_geometry <out_dir> [files]\n");
        return 1;
    }
    // "files": also run the reference's own grid_layout writer (cylinder_helpers.cuh:388-470)
    // with <out_dir> as the working directory, where it writes OUTPUT/CYLINDER/<ID_SIM>/grid_layout/
    const bool files = argc > 2 && std::string(argv[2]) == "files";
    const std::string out = argv[1];
    nodeVar h{};
    h.nodeType = (nodeType_t *)calloc(NUM_LBM_NODES, sizeof(nodeType_t));
    initialize_nodeType(h);
    boundaryVar b{};
    if (triangular) initialize_cylinder_nodeType_triangular(h, b);
    else initialize_cylinder_nodeType_staircase(h, b);
    b.boundaryList = (size_t *)malloc(b.NB * sizeof(size_t));
    b.incomingMask = (uint32_t *)malloc(b.NB * sizeof(uint32_t));
    b.outgoingMask = (uint32_t *)malloc(b.NB * sizeof(uint32_t));
    b.unit_nx = (real *)malloc(b.NB * sizeof(real));
    b.unit_ny = (real *)malloc(b.NB * sizeof(real));
    b.delta_w = (real *)malloc(b.NB * sizeof(real));
    b.bcfluidList = (size_t *)malloc((b.NB_FLUID > 0 ? b.NB_FLUID : 1) * sizeof(size_t));
#if Z_PERIODIC
    b.NB_SOLID = 0;  // only classified without z periodicity
#endif
    b.bcsolidList = (size_t *)malloc((b.NB_SOLID > 0 ? b.NB_SOLID : 1) * sizeof(size_t));
    buildBoundaryList_updateBoundaryNodeType(h, b, NODE_INNER, NODE_BCFLUID_INNER, NODE_BCSOLID_INNER);
    assignBoundaryIndices(h, b, NODE_INNER);
    compute_unit_vectors_boundary_nodes(h, b, D_WALL);
    find_incomings_outgoings(h, b);
    if (triangular) {
        setup_bcfluid_masks(h, b);
        setup_bcsolid_masks(h, b);
    }

    const int meta[8] = {NX, NY, NZ, b.NB, b.NB_FLUID, b.NB_SOLID, Z_PERIODIC, 0};
    const float fmeta[4] = {XC, YC, D_WALL, (float)OMEGA};
    dump(out, "meta.i32", meta, sizeof(meta));
    dump(out, "meta.f32", fmeta, sizeof(fmeta));
    dump(out, "node_type_tiled.u32", h.nodeType, NUM_LBM_NODES * sizeof(nodeType_t));
    dump(out, "boundary_list_tiled.u64", b.boundaryList, b.NB * sizeof(size_t));
    dump(out, "unit_nx.f32", b.unit_nx, b.NB * sizeof(real));
    dump(out, "unit_ny.f32", b.unit_ny, b.NB * sizeof(real));
    dump(out, "delta_w.f32", b.delta_w, b.NB * sizeof(real));
    dump(out, "in_mask.u32", b.incomingMask, b.NB * sizeof(uint32_t));
    dump(out, "out_mask.u32", b.outgoingMask, b.NB * sizeof(uint32_t));
    dump(out, "bcfluid_list_tiled.u64", b.bcfluidList, b.NB_FLUID * sizeof(size_t));
    dump(out, "tag_in_mask.u32", h_incomingMask_bcfluid, sizeof(h_incomingMask_bcfluid));
    dump(out, "tag_out_mask.u32", h_outgoingMask_bcfluid, sizeof(h_outgoingMask_bcfluid));
    dump(out, "bcsolid_list_tiled.u64", b.bcsolidList, b.NB_SOLID * sizeof(size_t));
    if (files) {
        if (chdir(out.c_str()) != 0) {
            fprintf(stderr, "cannot enter %s\n", out.c_str());
            return 2;
        }
        std::filesystem::create_directories(construct_path(PATH_FILES, ID_SIM, "grid_layout"));
        write_geometry_files(h);
    }
    printf("NB=%d NB_FLUID=%d NB_SOLID=%d\n", b.NB, b.NB_FLUID, b.NB_SOLID);
    return 0;
}
