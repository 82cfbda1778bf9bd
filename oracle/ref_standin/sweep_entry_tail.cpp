    return loc_norm;
}

extern "C" {

static const int ref_face_verts[4][3] = {{0, 1, 3}, {1, 2, 3}, {2, 0, 3}, {0, 2, 1}};  // VTK tetra faces

static void ref_vertex_matrices(int N, const double* vert, std::vector<Matrix4>& vertexs)
{
    // SetVertexMatrix (utils/grid_geometry/geometry_data.cpp:453-469): column j = vertex j, row 3 = 1
    vertexs.assign(N, Matrix4());
    for (int c = 0; c < N; ++c)
        for (int j = 0; j < 4; ++j) {
            for (int i = 0; i < 3; ++i) vertexs[c](i, j) = vert[12 * c + 3 * j + i];
            vertexs[c](3, j) = 1;
        }
}

// MakeArrayX on the mesh: nodes [N][4][3][3]
int ref_sweep_nodes(int N, const double* vert, double* nodes)
{
    std::vector<Matrix4> vertexs;
    ref_vertex_matrices(N, vert, vertexs);
    std::vector<BasePointTetra> vec_x(N);
    if (MakeArrayX(vertexs, vec_x)) return -1;
    for (int c = 0; c < N; ++c)
        for (int f = 0; f < base; ++f)
            for (int n = 0; n < 3; ++n)
                for (int i = 0; i < 3; ++i) nodes[36 * c + 9 * f + 3 * n + i] = vec_x[c].x[f][n][i];
    return 0;
}

// One direction: build_graph's order (as build_graph_main.cpp:165-300 drives
// it, without inner boundaries), then make_illum_struct's face states and
// LocX0 records (struct_short_characteristics_main.cpp:128-150).  Returns
// the record count, or < 0 on failure.
long long ref_sweep_structs(int N, const double* vert, const int* pairs_in, const double* normals_in,
                            const double* dir_in, int* graph_out, int* states_out, double* s_out,
                            unsigned char* face_out, int* nsteps_out)
{
    ref_failed = 0;
    std::vector<Normals> normals(N);
    std::vector<Face> grid((size_t)N * 4);
    for (int c = 0; c < N; ++c)
        for (int f = 0; f < 4; ++f) {
            const double* n = normals_in + 12 * c + 3 * f;
            normals[c].n[f] = Vector3(n[0], n[1], n[2]);
            const double* a = vert + 12 * c + 3 * ref_face_verts[f][0];
            const double* b = vert + 12 * c + 3 * ref_face_verts[f][1];
            const double* d = vert + 12 * c + 3 * ref_face_verts[f][2];
            grid[4 * c + f].A = Vector3(a[0], a[1], a[2]);
            grid[4 * c + f].B = Vector3(b[0], b[1], b[2]);
            grid[4 * c + f].C = Vector3(d[0], d[1], d[2]);
        }
    std::vector<Matrix4> vertexs;
    ref_vertex_matrices(N, vert, vertexs);
    std::vector<IntId> all_pairs(pairs_in, pairs_in + (size_t)N * 4);
    const Vector3 direction(dir_in[0], dir_in[1], dir_in[2]);

    std::vector<State> faces_state;
    std::map<IntId, FaceCell> inner_faces;
    InitFacesState(all_pairs, faces_state, inner_faces);
    std::vector<IntId> count_in_face, count_knew_face, cur_el;
    std::set<IntId> next_step_el;
    FindNumberOfAllInnerFaceAndKnew(direction, normals, faces_state, count_in_face, count_knew_face, next_step_el);
    int count_graph = 0, steps = 0;
    while (next_step_el.size()) {
        if (FindCurCell(next_step_el, count_in_face, count_knew_face, cur_el) == -1) return -1;
        NewStep(all_pairs, count_in_face, count_knew_face, cur_el, next_step_el);
        for (auto el : cur_el) graph_out[count_graph++] = el;
        ++steps;
    }
    if (count_graph != N) return -1;

    std::vector<BasePointTetra> vec_x(N);
    if (MakeArrayX(vertexs, vec_x)) return -2;
    std::vector<cell_local> vec_x0;
    std::vector<Type> vec_res_bound;
    for (int h = 0; h < N; ++h) {
        const int num_cell = graph_out[h];
        int face_state = 0;
        GetInAndOutFaces(direction, normals[num_cell], face_state);
        states_out[num_cell] = face_state;
        for (ShortId f = 0; f < base; ++f)
            if (!check_bit(face_state, f))
                GetNodes(num_cell, grid, f, vertexs[num_cell], face_state, direction, normals, all_pairs,
                         vec_x[num_cell], vec_res_bound, vec_x0);
    }
    if (ref_failed) return -3;
    for (size_t r = 0; r < vec_x0.size(); ++r) {
        s_out[r] = vec_x0[r].s;
        face_out[r] = vec_x0[r].in_face_id;
    }
    *nsteps_out = steps;
    return (long long)vec_x0.size();
}

}  // extern "C"
