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

// GetSend / GetDisp
void ref_get_send_disp(int np, int n, int* send_out, int* disp_out)
{
    std::vector<int> s, d;
    GetSend(np, n, s);
    GetDisp(np, n, d);
    for (int i = 0; i < np; ++i) { send_out[i] = s[i]; disp_out[i] = d[i]; }
}

}  // extern "C"
