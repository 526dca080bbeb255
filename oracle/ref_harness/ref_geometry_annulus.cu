// Geometry pin for the annulus: drives the reference's own host-side node classification
// (sakthi-lbm/MRLBM_3D_CUDA, shipped annulus case, compiled with CASE_ID = CASE_ANNULUS) and
// dumps it for both walls (and the BCSOLID lists of a Z_PERIODIC 0 build), so the oracle's
// and the product's restatements can be checked against it.  Test infrastructure only; no GPU is used: the calls follow
// cases/annulus/annulus_kernels.cu:5-49 (annulus_initialize) on malloc'd arrays.
#include <cstdio>
#include <cstdlib>
#include <string>

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

static void alloc_wall(boundaryVar &b) {
    b.boundaryList = (size_t *)malloc(b.NB * sizeof(size_t));
    b.incomingMask = (uint32_t *)malloc(b.NB * sizeof(uint32_t));
    b.outgoingMask = (uint32_t *)malloc(b.NB * sizeof(uint32_t));
    b.unit_nx = (real *)malloc(b.NB * sizeof(real));
    b.unit_ny = (real *)malloc(b.NB * sizeof(real));
    b.delta_w = (real *)malloc(b.NB * sizeof(real));
    b.bcfluidList = (size_t *)malloc((b.NB_FLUID > 0 ? b.NB_FLUID : 1) * sizeof(size_t));
#if Z_PERIODIC
    b.NB_SOLID = 0;
#endif
    b.bcsolidList = (size_t *)malloc((b.NB_SOLID > 0 ? b.NB_SOLID : 1) * sizeof(size_t));
}

static void dump_wall(const std::string &out, const char *tag, const boundaryVar &b) {
    auto name = [&](const char *what) { return std::string(tag) + "_" + what; };
    dump(out, name("boundary_list_tiled.u64").c_str(), b.boundaryList, b.NB * sizeof(size_t));
    dump(out, name("unit_nx.f32").c_str(), b.unit_nx, b.NB * sizeof(real));
    dump(out, name("unit_ny.f32").c_str(), b.unit_ny, b.NB * sizeof(real));
    dump(out, name("delta_w.f32").c_str(), b.delta_w, b.NB * sizeof(real));
    dump(out, name("in_mask.u32").c_str(), b.incomingMask, b.NB * sizeof(uint32_t));
    dump(out, name("out_mask.u32").c_str(), b.outgoingMask, b.NB * sizeof(uint32_t));
    dump(out, name("bcfluid_list_tiled.u64").c_str(), b.bcfluidList, b.NB_FLUID * sizeof(size_t));
    dump(out, name("bcsolid_list_tiled.u64").c_str(), b.bcsolidList, b.NB_SOLID * sizeof(size_t));
}

int main(int argc, char **argv) {
    if (argc < 2) {
        fprintf(stderr, "usage: ref_geometry_annulus <out_dir>\n");
        return 1;
    }
    const std::string out = argv[1];
    nodeVar h{};
    h.nodeType = (nodeType_t *)calloc(NUM_LBM_NODES, sizeof(nodeType_t));
    initialize_nodeType(h);
    boundaryVar in{}, outer{};
    initialize_annulus_nodeType_triangular(h, in, outer);
    alloc_wall(in);
    alloc_wall(outer);
    buildBoundaryList_updateBoundaryNodeType(h, in, NODE_INNER, NODE_BCFLUID_INNER, NODE_BCSOLID_INNER);
    buildBoundaryList_updateBoundaryNodeType(h, outer, NODE_OUTER, NODE_BCFLUID_OUTER, NODE_BCSOLID_OUTER);
    assignBoundaryIndices(h, in, NODE_INNER);
    assignBoundaryIndices(h, outer, NODE_OUTER);
    compute_unit_vectors_boundary_nodes(h, in, D_IN);
    compute_unit_vectors_boundary_nodes(h, outer, D_OUT);
    find_incomings_outgoings(h, in);
    find_incomings_outgoings(h, outer);
    setup_bcfluid_masks(h, in);
    setup_bcfluid_masks(h, outer);

    const int meta[10] = {NX, NY, NZ, in.NB, in.NB_FLUID, outer.NB, outer.NB_FLUID, in.NB_SOLID, outer.NB_SOLID,
                          Z_PERIODIC};
    dump(out, "meta.i32", meta, sizeof(meta));
    dump(out, "node_type_tiled.u32", h.nodeType, NUM_LBM_NODES * sizeof(nodeType_t));
    dump_wall(out, "inner", in);
    dump_wall(out, "outer", outer);
    dump(out, "tag_in_mask.u32", h_incomingMask_bcfluid, sizeof(h_incomingMask_bcfluid));
    dump(out, "tag_out_mask.u32", h_outgoingMask_bcfluid, sizeof(h_outgoingMask_bcfluid));
    printf("NB=%d/%d NB_FLUID=%d/%d\n", in.NB, outer.NB, in.NB_FLUID, outer.NB_FLUID);
    return 0;
}
