/* A plain C client of libdecaes_gpu.so: what a foreign caller (Julia ccall,
 * cgo, JNI) does through include/decaes_gpu.h, limited to the entry points
 * that need no GPU.  Built and run by tests/test_c_abi.py, as C99 and as C++.
 *
 * Output, one item per line:
 *   t2map_valid <rc>
 *   t2map_invalid <rc> <message>
 *   t2part_valid <rc>
 *   t2part_invalid <rc> <message>
 *   mock <rc>      and the image bytes written to the file named by argv[1]
 */
#include <math.h>
#include <stdio.h>
#include <string.h>

#include "decaes_gpu.h"

int main(int argc, char **argv) {
    char msg[512];
    decaes_t2map_opts o;
    decaes_t2part_opts p;
    decaes_mock_opts mo;
    double img[4 * 3 * 2 * 32];
    FILE *f;
    int rc;

    if (argc != 2) return 2;
    memset(&o, 0, sizeof o);
    o.MatrixSize[0] = 4; o.MatrixSize[1] = 3; o.MatrixSize[2] = 2;
    o.nTE = 32; o.TE = 10e-3; o.nT2 = 40; o.T2Range[0] = 10e-3; o.T2Range[1] = 2.0;
    o.T1 = 1.0; o.Threshold = 0.0; o.MinRefAngle = 50.0; o.nRefAngles = 8; o.nRefAnglesMin = 5;
    o.Reg = DECAES_REG_CHI2; o.Chi2Factor = 1.02; o.NoiseLevel = NAN; o.RefConAngle = 180.0;
    o.SetFlipAngle = NAN; o.precision = DECAES_PREC_FP64;
    rc = decaes_t2map_check_options(&o, msg, sizeof msg);
    printf("t2map_valid %d\n", rc);
    o.Chi2Factor = 0.5;
    rc = decaes_t2map_check_options(&o, msg, sizeof msg);
    printf("t2map_invalid %d %s\n", rc, msg);

    memset(&p, 0, sizeof p);
    p.MatrixSize[0] = 4; p.MatrixSize[1] = 3; p.MatrixSize[2] = 2;
    p.nT2 = 40; p.T2Range[0] = 10e-3; p.T2Range[1] = 2.0;
    p.SPWin[0] = 10e-3; p.SPWin[1] = 25e-3; p.MPWin[0] = 25e-3; p.MPWin[1] = 200e-3; p.Sigmoid = NAN;
    rc = decaes_t2part_check_options(&p, msg, sizeof msg);
    printf("t2part_valid %d\n", rc);
    p.SPWin[0] = 30e-3;
    rc = decaes_t2part_check_options(&p, msg, sizeof msg);
    printf("t2part_invalid %d %s\n", rc, msg);

    memset(&mo, 0, sizeof mo);
    mo.MatrixSize[0] = 4; mo.MatrixSize[1] = 3; mo.MatrixSize[2] = 2;
    mo.nTE = 32; mo.TE = 10e-3; mo.T1 = 1.0;
    mo.FlipAngleRange[0] = 140.0; mo.FlipAngleRange[1] = 180.0;
    mo.MyelinT2Range[0] = 15e-3; mo.MyelinT2Range[1] = 25e-3;
    mo.MyelinFracRange[0] = 0.05; mo.MyelinFracRange[1] = 0.25;
    mo.IET2Range[0] = 60e-3; mo.IET2Range[1] = 90e-3;
    mo.CSFT2Range[0] = 1.0; mo.CSFT2Range[1] = 2.0;
    mo.CSFFracRange[0] = 0.0; mo.CSFFracRange[1] = 0.05;
    mo.AmplitudeRange[0] = 500.0; mo.AmplitudeRange[1] = 2000.0;
    mo.SNRRange[0] = 50.0; mo.SNRRange[1] = 200.0;
    mo.BackgroundFraction = 0.0; mo.BackgroundSigma = 8.0;
    rc = decaes_mock_image(&mo, 11, img, DECAES_F64, 2);
    printf("mock %d\n", rc);
    f = fopen(argv[1], "wb");
    if (!f) return 3;
    if (fwrite(img, sizeof img, 1, f) != 1) { fclose(f); return 4; }
    fclose(f);
    return 0;
}
