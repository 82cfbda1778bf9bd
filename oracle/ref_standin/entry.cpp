// entry.cpp -- extern "C" wrappers appended after the reference's own
// function text by oracle/build_ref.sh.  TEST INFRASTRUCTURE ONLY.
extern "C" {

static void ref_fill_dirs(grid_directions_t& gd, int M, const double* xyz,
                          const double* area, double full_area)
{
    gd.size = M;
    gd.directions.resize(M);
    for (int i = 0; i < M; ++i) {
        gd.directions[i].dir = Vector3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
        gd.directions[i].area = area[i];
    }
    gd.full_area = full_area;
}

// CalculateIntCPU over out-directions [disp_loc, disp_loc + size_loc)
int ref_calculate_int_cpu(int N, int M, const double* xyz, const double* area,
                          double full_area, double* illum, int disp_loc, int size_loc,
                          double* scattering)
{
    grid_directions_t gd;
    ref_fill_dirs(gd, M, xyz, area, full_area);
    grid_t g;
    g.size = N;
    g.Illum = illum;
    g.scattering = scattering;
    disp.assign(1, disp_loc);
    send_count.assign(1, size_loc);
    return CalculateIntCPU(N, gd, g);
}

// IntegarteDirection (energy) for one cell; illum_cell is [M][4]
double ref_energy_cell(int M, const double* xyz, const double* area, double full_area,
                       const double* illum_cell)
{
    grid_directions_t gd;
    ref_fill_dirs(gd, M, xyz, area, full_area);
    std::vector<Type> I(illum_cell, illum_cell + (size_t)M * base);
    return IntegarteDirection(I, gd);
}

// IntegarteDirection3 + the face mean of MakeStream for one cell
void ref_stream_cell(int M, const double* xyz, const double* area, double full_area,
                     const double* illum_cell, double* out3)
{
    grid_directions_t gd;
    ref_fill_dirs(gd, M, xyz, area, full_area);
    std::vector<Type> I(illum_cell, illum_cell + (size_t)M * base);
    Vector3 Stream[base];
    IntegarteDirection3(I, gd, Stream);
    Vector3 s;
    GET_FACE_TO_CELL(s, Stream, Vector3::Zero());
    out3[0] = s[0];
    out3[1] = s[1];
    out3[2] = s[2];
}

// MakeStream + MakeDivImpuls on N cells: illum [M][N][4] (the GPU layout,
// regrouped per cell as the CPU code keeps it), per-cell outward normals
// [N][4][3], face areas [N][4], volumes [N].  Each (cell, face) gets its own
// face record with sign_n = true.  Outputs: flux [N][3], impuls [N][9]
// (row-major), divstream [N], divimpuls [N][3].
void ref_illum_params(int N, int M, const double* xyz, const double* area, double full_area,
                      const double* illum, const double* normals, const double* face_areas,
                      const double* volume, double* flux, double* impuls, double* divstream,
                      double* divimpuls)
{
    grid_directions_t gd;
    ref_fill_dirs(gd, M, xyz, area, full_area);
    grid_t g;
    g.size = N;
    g.Illum = nullptr;
    g.scattering = nullptr;
    g.cells.resize(N);
    g.faces.resize((size_t)N * base);
    for (int c = 0; c < N; ++c) {
        elem_t& el = g.cells[c];
        el.illum_val.illum.resize((size_t)M * base);
        for (int j = 0; j < M; ++j)
            for (int f = 0; f < base; ++f)
                el.illum_val.illum[(size_t)j * base + f] = illum[((size_t)j * N + c) * base + f];
        el.geo.V = volume[c];
        for (int f = 0; f < base; ++f) {
            const size_t id = (size_t)c * base + f;
            el.geo.id_faces[f] = (int)id;
            el.geo.sign_n[f] = true;
            g.faces[id].geo.n = Vector3(normals[3 * id], normals[3 * id + 1], normals[3 * id + 2]);
            g.faces[id].geo.S = face_areas[id];
        }
    }
    MakeStream(gd, g);
    MakeDivImpuls(gd, g);
    for (int c = 0; c < N; ++c) {
        const illum_value_t& v = g.cells[c].illum_val;
        for (int h = 0; h < 3; ++h) {
            flux[3 * c + h] = v.stream[h];
            divimpuls[3 * c + h] = v.div_impuls[h];
            for (int k = 0; k < 3; ++k) impuls[9 * c + 3 * h + k] = v.impuls(h, k);
        }
        divstream[c] = v.div_stream;
    }
}

// GetSend / GetDisp
void ref_get_send_disp(int np, int n, int* send_out, int* disp_out)
{
    std::vector<int> s, d;
    GetSend(np, n, s);
    GetDisp(np, n, d);
    for (int i = 0; i < np; ++i) { send_out[i] = s[i]; disp_out[i] = d[i]; }
}

}  // extern "C"
