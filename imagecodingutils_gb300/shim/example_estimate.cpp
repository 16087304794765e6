// example_estimate.cpp -- how a vpp codec drives the GPU classes.
//
//   example_estimate <pair.bin> <width> <height> <motionRange> <out.bin> [estimator]
//
// pair.bin holds the source then the reference luma plane (int16).  The
// program estimates with GpuMotionEstimatorH264ImplFull (or, by the optional
// last argument, ...Multires, ...MultiresCross, ...MultiresCrossVer2 or
// ...Cross, ...UMHS, ...FHS, H263ImplMultiresCrossVer2: "multires", "mrc", "mrc2", "cross", "sad", "umhs", "h263mrc2",
// "fhs"; "impl1" / "impl2" are MotionEstimatorImpl1 / Impl2 with 16x16 blocks, a +-16 pel range and SetMode(0),
// its half-pel char vectors widened to the output's shorts; "mrc2lam" is Ver2's Lagrangian Estimate(long*, void*) with lambda 2.5;
// UMHS gets the previous frame's vectors from a first estimate of the same
// pair, as a codec chains frames) exactly as a codec would
// with the vpp class (constructor, Create, SetMode(0), Estimate, predictor
// side effect), then
// runs the forward/inverse 4x4 transform classes
// on the motion-compensated-free residual (source - reference) of the first
// macroblock row, and the Intra16x16-style DC path (4x4 transform only, DC
// gathered per macroblock, DC Hadamard + quantisation and inverse) on it.
// out.bin receives: the vectors (N x 2 int16), avgDistortion (int64), the
// predictor's copy of the vectors (N x 2 int32), the transformed residual
// levels and reconstruction (int16), then the DC levels and the inverse DC
// (int16, 16 per macroblock of the row).
#include <stdio.h>
#include <stdlib.h>
#include <string>
#include <vector>

#include "vppgpu_vpp.hpp"

class RecordingPredictor : public IMotionVectorPredictor {
public:
    explicit RecordingPredictor(int n) : mv(2 * (size_t)n, 0) {}
    virtual int Create(void) { return 1; }
    virtual int Get16x16Prediction(void*, int, int* x, int* y) { *x = *y = 0; return 1; }
    virtual void Set16x16MotionVector(int blk, int x, int y) { mv[2 * blk] = x; mv[2 * blk + 1] = y; }
    virtual void Set16x16MotionVector(int blk, int x, int y, int d)
    {
        Set16x16MotionVector(blk, x, y);
        if ((size_t)blk < dist.size()) dist[blk] = d;
    }
    std::vector<int> mv;
    std::vector<int> dist;
};

int main(int argc, char** argv)
{
    if (argc != 6 && argc != 7) {
        fprintf(stderr, "usage: %s pair.bin width height motionRange out.bin "
                        "[full|multires|mrc|mrc2|mrc2lam|h263mrc2|cross|sad|umhs|fhs|impl1|impl2]\n", argv[0]);
        return 2;
    }
    const std::string kind = argc == 7 ? argv[6] : "full";
    int w = atoi(argv[2]), h = atoi(argv[3]), range = atoi(argv[4]);
    std::vector<short> src((size_t)w * h), ref((size_t)w * h);
    FILE* f = fopen(argv[1], "rb");
    if (!f || fread(src.data(), 2, src.size(), f) != src.size() || fread(ref.data(), 2, ref.size(), f) != ref.size())
        return 3;
    fclose(f);
    int nmb = (w / 16) * (h / 16);
    bool* incl = new bool[nmb];
    for (int i = 0; i < nmb; i++) incl[i] = true;

    RecordingPredictor pred(nmb);
    pred.dist.assign(nmb, -1);
    if (kind == "impl1" || kind == "impl2") {  // no predictor: the vectors and the average only
        GpuMotionEstimatorImpl1* me1 = kind == "impl1"
                                           ? new GpuMotionEstimatorImpl1(src.data(), ref.data(), w, h, 16, 16, 16)
                                           : new GpuMotionEstimatorImpl2(src.data(), ref.data(), w, h, 16, 16, 16);
        if (!me1->Create()) return 4;
        me1->SetMode(0);
        long a1 = 0;
        SimpleMotionVectorList* l = (SimpleMotionVectorList*)me1->Estimate(&a1);
        if (!l) return 5;
        FILE* o1 = fopen(argv[5], "wb");
        const signed char* p = (const signed char*)l->GetDataPtr();
        for (int k = 0; k < l->GetLength(); k++) {
            short v[2] = {(short)p[(size_t)k * l->GetPatternSize()], (short)p[(size_t)k * l->GetPatternSize() + 1]};
            fwrite(v, 2, 2, o1);
        }
        long long a = a1;
        fwrite(&a, 8, 1, o1);
        fclose(o1);
        delete me1;
        delete[] incl;
        return 0;
    }
    std::vector<short> prev_mv;
    IMotionEstimator* me;
    if (kind == "multires")
        me = new GpuMotionEstimatorH264ImplMultires(src.data(), ref.data(), w, h, range, &pred, incl);
    else if (kind == "mrc")
        me = new GpuMotionEstimatorH264ImplMultiresCross(src.data(), ref.data(), w, h, range, incl);
    else if (kind == "h263mrc2")  // half-pel range 64: the same +-31 pels as the quarter-pel 128
        me = new GpuMotionEstimatorH263ImplMultiresCrossVer2(src.data(), ref.data(), w, h, range / 2, &pred, incl);
    else if (kind == "mrc2" || kind == "mrc2lam")
        me = new GpuMotionEstimatorH264ImplMultiresCrossVer2(src.data(), ref.data(), w, h, range, &pred, incl);
    else if (kind == "cross")
        me = new GpuMotionEstimatorH264ImplCross(src.data(), ref.data(), w, h, range, &pred, incl);
    else if (kind == "sad")
        me = new GpuMotionEstimatorH264ImplFullSad(src.data(), ref.data(), w, h, range, &pred, incl);
    else if (kind == "umhs") {
        // a first estimate without a previous frame gives the vectors the second one starts from
        GpuMotionEstimatorH264ImplUMHS first(src.data(), ref.data(), w, h, range, NULL);
        long a0 = 0;
        VectorStructList* v0 = first.Create() ? (VectorStructList*)first.Estimate(&a0) : NULL;
        if (!v0) return 6;
        prev_mv.resize(2 * (size_t)nmb);
        for (int k = 0; k < nmb; k++) {
            prev_mv[2 * k] = (short)v0->GetSimpleElement(k, 0);
            prev_mv[2 * k + 1] = (short)v0->GetSimpleElement(k, 1);
        }
        GpuMotionEstimatorH264ImplUMHS* u = new GpuMotionEstimatorH264ImplUMHS(src.data(), ref.data(), w, h, range,
                                                                               &pred, incl);
        u->SetPrevFrame(prev_mv.data(), NULL);
        me = u;
    } else if (kind == "fhs")
        me = new GpuMotionEstimatorH264ImplFHS(src.data(), ref.data(), w, h, range, &pred, incl);
    else
        me = new GpuMotionEstimatorH264ImplFull(src.data(), ref.data(), w, h, range, &pred, incl);
    if (!me->Create()) {
        fprintf(stderr, "Create failed\n");
        return 4;
    }
    me->SetMode(0);
    long avg = 0;
    double lambda = 2.5;
    VectorStructList* vl =
        (VectorStructList*)(kind == "mrc2lam" ? me->Estimate(&avg, (void*)&lambda) : me->Estimate(&avg));
    if (!vl) {
        fprintf(stderr, "Estimate failed\n");
        return 5;
    }

    // residual of the first macroblock row, 4x4 blocks laid out contiguously
    int nblk = (w / 4) * 4;
    std::vector<short> blocks(16 * (size_t)nblk);
    for (int b = 0; b < nblk; b++)
        for (int r = 0; r < 4; r++)
            for (int c = 0; c < 4; c++) {
                int y = (b / (w / 4)) * 4 + r, x = (b % (w / 4)) * 4 + c;
                blocks[16 * b + 4 * r + c] = (short)(src[(size_t)y * w + x] - ref[(size_t)y * w + x]);
            }
    GpuForward4x4IT fwd;
    fwd.SetParameter(IForwardTransform::INTRA_FLAG_ID, 0);
    fwd.SetParameter(IForwardTransform::QUANT_ID, 28);
    std::vector<short> levels_src = blocks;
    fwd.TransformBlocks(blocks.data(), nblk);
    std::vector<short> levels = blocks;
    GpuInverse4x4IT inv;
    inv.SetParameter(IInverseTransform::QUANT_ID, 28);
    inv.InverseTransformBlocks(blocks.data(), nblk);

    // Intra16x16-style DC path on the same residual: 4x4 transform only, the
    // 16 DC coefficients of each macroblock gathered into a 4x4 block, then the
    // DC Hadamard with quantisation and its inverse
    std::vector<short> coeffs(16 * (size_t)nblk);
    for (int b = 0; b < nblk; b++)
        for (int i = 0; i < 16; i++) coeffs[16 * b + i] = levels_src[16 * b + i];
    GpuForward4x4IT it_only;
    it_only.SetMode(IForwardTransform::TransformOnly);
    it_only.TransformBlocks(coeffs.data(), nblk);
    const int nmbr = w / 16;
    std::vector<short> dc(16 * (size_t)nmbr);
    for (int m = 0; m < nmbr; m++)
        for (int r = 0; r < 4; r++)
            for (int c = 0; c < 4; c++) dc[16 * m + 4 * r + c] = coeffs[16 * (r * (w / 4) + 4 * m + c)];
    GpuForwardDCIT fdc(4);
    fdc.SetParameter(IForwardTransform::QUANT_ID, 28);
    fdc.TransformBlocks(dc.data(), nmbr);
    std::vector<short> dc_levels = dc;
    GpuInverseDCIT idc(4);
    idc.SetParameter(IInverseTransform::QUANT_ID, 28);
    idc.InverseTransformBlocks(dc.data(), nmbr);

    FILE* o = fopen(argv[5], "wb");
    for (int k = 0; k < nmb; k++) {
        short v[2] = {(short)vl->GetSimpleElement(k, 0), (short)vl->GetSimpleElement(k, 1)};
        fwrite(v, 2, 2, o);
    }
    long long a = avg;
    fwrite(&a, 8, 1, o);
    fwrite(pred.mv.data(), 4, pred.mv.size(), o);
    fwrite(levels.data(), 2, levels.size(), o);
    fwrite(blocks.data(), 2, blocks.size(), o);
    fwrite(dc_levels.data(), 2, dc_levels.size(), o);
    fwrite(dc.data(), 2, dc.size(), o);
    fwrite(pred.dist.data(), 4, pred.dist.size(), o);
    fwrite(prev_mv.data(), 2, prev_mv.size(), o);
    fclose(o);
    delete me;
    delete[] incl;
    return 0;
}
