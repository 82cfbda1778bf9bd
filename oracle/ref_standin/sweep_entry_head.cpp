// sweep_entry_head.cpp / sweep_entry_tail.cpp -- the harness around the
// reference's own sweep loop (solve_module/illum/Illum_async.cpp:726-784),
// which oracle/build_ref.sh places between the two files, plus extern "C"
// entry points for the reference's cell ordering (build_graph) and
// characteristic geometry (make_illum_struct).  TEST INFRASTRUCTURE ONLY.
// One sweep of directions [0, ndir) as MPI_CalculateIllumAsync's first
// direction loop runs it on one rank: the containers are filled from flat
// arrays with the reference's names, then the loop text follows.
extern "C" double ref_sweep_dirs(int count_cells, int ndir, const int* pairs_in, const int* order_in,
                                 const int* states_in, const long long* rec_off, const double* rec_s,
                                 const unsigned char* rec_face, const double* nodes, const double* scattering,
                                 int class_vtk, const double* density, const double* pressure, double* illum)
{
    solve_mode.class_vtk = class_vtk;
    const int size_1_section = ndir;
    const int myid = 0;
    std::vector<int> disp_illum(1, 0);
    std::vector<int> pairs(pairs_in, pairs_in + (size_t)count_cells * base);
    std::vector<std::vector<int>> sorted_id_cell(ndir), face_states(ndir);
    std::vector<std::vector<cell_local>> vec_x0(ndir);
    for (int d = 0; d < ndir; ++d) {
        sorted_id_cell[d].assign(order_in + (size_t)d * count_cells, order_in + (size_t)(d + 1) * count_cells);
        face_states[d].assign(states_in + (size_t)d * count_cells, states_in + (size_t)(d + 1) * count_cells);
        for (long long r = rec_off[d]; r < rec_off[d + 1]; ++r) {
            cell_local c;
            c.s = rec_s[r];
            c.x0 = Vector2(0, 0);
            c.in_face_id = rec_face[r];
            vec_x0[d].push_back(c);
        }
    }
    std::vector<BasePointTetra> vec_x(count_cells);
    for (int c = 0; c < count_cells; ++c)
        for (int f = 0; f < base; ++f)
            for (int n = 0; n < 3; ++n)
                vec_x[c].x[f][n] = Vector3(nodes[36 * c + 9 * f + 3 * n], nodes[36 * c + 9 * f + 3 * n + 1],
                                           nodes[36 * c + 9 * f + 3 * n + 2]);
    phys_local.assign(count_cells, flux_t{});
    if (density && pressure)
        for (int c = 0; c < count_cells; ++c) phys_local[c].d = density[c], phys_local[c].p = pressure[c];
    grid_t grid;
    grid.size = count_cells;
    grid.Illum = illum;
    grid.scattering = const_cast<double*>(scattering);
    std::vector<Vector3> inter_coef_store((size_t)count_cells * base);
    std::vector<Vector3>* inter_coef = &inter_coef_store;
    Type loc_norm = -1;
