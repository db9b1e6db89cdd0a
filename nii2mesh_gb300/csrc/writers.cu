// writers.cu — the mesh file formats of save_mesh() (src/meshify.c:984-1019)
// assembled in device memory: mz3 (plain or gzip, :602-679), GIfTI (base64,
// or zlib + base64, :819-930), FreeSurfer (:418-459), JSON (:683-698), OFF
// (:700-711), OBJ (:713-723), STL (:725-762), PLY (:764-817) and VTK
// (:932-971).  Every byte equals the reference writer's output (the GPU
// deflate differs from zlib's; its decompressed bytes are equal).
//
// Binary sections are packed by one thread per vertex / triangle straight
// from the ABI mesh (vec3d -> float32 rounded to nearest, byte-swapped where
// the reference swaps); text lines (%g / %d) are formatted one thread per
// line, in registers, into 48-byte slots, then scanned and compacted by warps.
#include <string.h>
#include <time.h>

#include "fmt.cuh"
#include "n2m_internal.cuh"

namespace {
__device__ __forceinline__ void put_u32(unsigned char *d, unsigned v, bool be) {
    if (be) {
        d[0] = (unsigned char)(v >> 24);
        d[1] = (unsigned char)(v >> 16);
        d[2] = (unsigned char)(v >> 8);
        d[3] = (unsigned char)v;
    } else {
        d[0] = (unsigned char)v;
        d[1] = (unsigned char)(v >> 8);
        d[2] = (unsigned char)(v >> 16);
        d[3] = (unsigned char)(v >> 24);
    }
}
__device__ __forceinline__ unsigned f32_bits(double v) { return (unsigned)__float_as_int(__double2float_rn(v)); }

// float32 vertices, 12 bytes each (be: byte-swapped as the reference's swap_4bytes)
__global__ void k_pack_pts(const vec3d *__restrict__ p, int np, unsigned char *__restrict__ dst, int be) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const vec3d v = p[i];
    unsigned char *d = dst + (size_t)12 * i;
    put_u32(d, f32_bits(v.x), be);
    put_u32(d + 4, f32_bits(v.y), be);
    put_u32(d + 8, f32_bits(v.z), be);
}

enum { TRI_LE12 = 0, TRI_BE12 = 1, TRI_PLY13 = 2, TRI_VTK16 = 3 };
__global__ void k_pack_tris(const vec3i *__restrict__ t, int nt, unsigned char *__restrict__ dst, int mode) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nt) return;
    const vec3i f = t[i];
    if (mode == TRI_PLY13) {   // uint8 3, int32 x3 little-endian, packed
        unsigned char *d = dst + (size_t)13 * i;
        d[0] = 3;
        put_u32(d + 1, (unsigned)f.x, false);
        put_u32(d + 5, (unsigned)f.y, false);
        put_u32(d + 9, (unsigned)f.z, false);
    } else if (mode == TRI_VTK16) {   // uint32 3, x, y, z big-endian
        unsigned char *d = dst + (size_t)16 * i;
        put_u32(d, 3u, true);
        put_u32(d + 4, (unsigned)f.x, true);
        put_u32(d + 8, (unsigned)f.y, true);
        put_u32(d + 12, (unsigned)f.z, true);
    } else {
        unsigned char *d = dst + (size_t)12 * i;
        const bool be = mode == TRI_BE12;
        put_u32(d, (unsigned)f.x, be);
        put_u32(d + 4, (unsigned)f.y, be);
        put_u32(d + 8, (unsigned)f.z, be);
    }
}

// binary STL facet: normal (0,0,0), three float32 corners, uint16 0 (50 bytes); a corner index
// outside [0, np) sets *bad and is written as the origin
__global__ void k_pack_stl(const vec3i *__restrict__ t, const vec3d *__restrict__ p, int nt, int np,
                           unsigned char *__restrict__ dst, unsigned *__restrict__ bad) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nt) return;
    const vec3i f = t[i];
    unsigned char *d = dst + (size_t)50 * i;
    for (int k = 0; k < 12; k++) d[k] = 0;
    const int idx[3] = {f.x, f.y, f.z};
    for (int c = 0; c < 3; c++) {
        vec3d v = {0.0, 0.0, 0.0};
        if ((unsigned)idx[c] < (unsigned)np) v = p[idx[c]];
        else atomicOr(bad, 1u);
        put_u32(d + 12 + 12 * c, f32_bits(v.x), false);
        put_u32(d + 16 + 12 * c, f32_bits(v.y), false);
        put_u32(d + 20 + 12 * c, f32_bits(v.z), false);
    }
    d[48] = d[49] = 0;
}

// base64 (RFC 4648 alphabet, '=' padding, no line breaks: base64_encode of src/base64.c without USE_EOLN)
__constant__ char c_b64[65] = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";
__global__ void k_base64(const unsigned char *__restrict__ in, long long n, unsigned char *__restrict__ out) {
    const long long g = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long i = 3 * g;
    if (i >= n) return;
    const unsigned b0 = in[i], b1 = i + 1 < n ? in[i + 1] : 0u, b2 = i + 2 < n ? in[i + 2] : 0u;
    unsigned char *o = out + 4 * g;
    o[0] = (unsigned char)c_b64[b0 >> 2];
    o[1] = (unsigned char)c_b64[((b0 & 3u) << 4) | (b1 >> 4)];
    o[2] = i + 1 < n ? (unsigned char)c_b64[((b1 & 15u) << 2) | (b2 >> 6)] : (unsigned char)'=';
    o[3] = i + 2 < n ? (unsigned char)c_b64[b2 & 63u] : (unsigned char)'=';
}

// one text line per vertex (%g) or triangle (%d of index + 1): pre num sep num sep num post,
// at most 48 characters, formatted in registers into the line's 48-byte slot
constexpr int SLOT = 48;
struct LineFmt {      // up to 4 characters each, first character in the low byte
    unsigned pre, sep, post;
    int npre, nsep, npost;
};
template <class S>
__device__ __forceinline__ void put_word(S &out, unsigned w, int n) {
    for (int j = 0; j < n; j++) out.put((char)(w >> (8 * j)));
}
template <bool TRI>
__global__ void k_txt_fmt(const void *__restrict__ src, int n, LineFmt f, unsigned *__restrict__ slots,
                          unsigned *__restrict__ lens) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    n2mfmt::WordSink out{slots + (size_t)(SLOT / 4) * i};
    put_word(out, f.pre, f.npre);
    for (int c = 0; c < 3; c++) {
        if (c) put_word(out, f.sep, f.nsep);
        if (TRI) n2mfmt::fmt_d(((const int *)src)[3 * (size_t)i + c] + 1, out);
        else n2mfmt::fmt_g6(((const double *)src)[3 * (size_t)i + c], out);
    }
    put_word(out, f.post, f.npost);
    out.done();
    lens[i] = (unsigned)out.n;
}

// slots -> the text: one warp per 32 lines; the 32 slots are staged in shared
// memory and the warp writes its contiguous output bytes lane by lane.
// offs: exclusive offsets (n + 1 entries)
constexpr int COPY_WARPS = 8;
__global__ void __launch_bounds__(32 * COPY_WARPS) k_txt_copy(const unsigned *__restrict__ slots,
                                                              const unsigned *__restrict__ offs, int n,
                                                              unsigned char *__restrict__ dst) {
    __shared__ unsigned sw[COPY_WARPS][32 * SLOT / 4];
    __shared__ unsigned so[COPY_WARPS][33];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long i0 = ((long long)blockIdx.x * COPY_WARPS + warp) * 32;
    if (i0 >= n) return;
    const int cnt = (int)min(32ll, n - i0);
    const unsigned *src = slots + (size_t)i0 * (SLOT / 4);
    for (int k = lane; k < cnt * (SLOT / 4); k += 32) sw[warp][k] = src[k];
    if (lane <= cnt) so[warp][lane] = offs[i0 + lane];
    if (lane == 0 && cnt == 32) so[warp][32] = offs[i0 + 32];
    __syncwarp();
    const unsigned end = so[warp][cnt];
    for (unsigned b = so[warp][0] + lane; b < end; b += 32) {
        int lo = 0, hi = cnt;   // so[lo] <= b < so[hi]
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (so[warp][mid] <= b) lo = mid;
            else hi = mid;
        }
        const unsigned off = b - so[warp][lo];
        dst[b] = (unsigned char)(sw[warp][lo * (SLOT / 4) + (off >> 2)] >> (8 * (off & 3)));
    }
}

unsigned grid(long long n, int b) { return (unsigned)((n + b - 1) / b); }

LineFmt line_fmt(const char *pre, const char *sep, const char *post) {
    auto pack = [](const char *t, int &n) {
        n = (int)strlen(t);
        unsigned w = 0;
        for (int j = 0; j < n; j++) w |= (unsigned)(unsigned char)t[j] << (8 * j);
        return w;
    };
    LineFmt f{};
    f.pre = pack(pre, f.npre);
    f.sep = pack(sep, f.nsep);
    f.post = pack(post, f.npost);
    return f;
}

struct Assembler {   // appends host text and device sections to w.out
    WriterWork &w;
    cudaStream_t s;
    size_t pos = 0;
    n2m_status text(const std::string &t) {
        if (t.empty()) return N2M_OK;
        CK(cudaMemcpyAsync(w.out.as<unsigned char>() + pos, t.data(), t.size(), cudaMemcpyHostToDevice, s));
        pos += t.size();
        return N2M_OK;
    }
};

std::string fmt_str(const char *f, long long a, long long b = 0) {
    char buf[128];
    snprintf(buf, sizeof buf, f, a, b);
    return buf;
}

// text format: lines of vertices then triangles between host text
n2m_status encode_text(int format, const vec3i *d_t, const vec3d *d_p, int nt, int np, WriterWork &w, ScanWork &sw,
                       cudaStream_t s, size_t *len) {
    LineFmt fv, ft;
    std::string head, mid, tail;
    if (format == N2M_FMT_OBJ) {
        fv = line_fmt("v ", " ", "\n");
        ft = line_fmt("f ", " ", "\n");
    } else if (format == N2M_FMT_OFF) {
        fv = ft = line_fmt("", " ", "\n");
        head = fmt_str("OFF\n%lld\t%lld\t0\n", np, nt);
    } else {   // JSON
        fv = ft = line_fmt("[", ",\t", "],\n");
        head = "{\n\t\"_DataInfo_\":{\n\t\t\"JMeshVersion\":\"0.5\",\n\t\t\"Comment\":\"Created by nii2mesh\"\n\t},\n"
               "\t\"MeshVertex3\":[\n";
        mid = "\t],\n\t\"MeshTri3\":[\n";
        tail = "\t]\n}\n";
    }
    const long long nl = (long long)np + nt;
    if ((unsigned long long)nl * SLOT >= (1ull << 32)) {
        n2m_set_error("text mesh too large for one file of < 4 GB");
        return N2M_ERR_TOO_LARGE;
    }
    CKS(w.pack.ensure((size_t)std::max<long long>(nl, 1) * SLOT));
    CKS(w.lens.ensure((size_t)(nl + 2) * sizeof(unsigned)));
    unsigned *slots = w.pack.as<unsigned>();
    unsigned *lens = w.lens.as<unsigned>();
    if (np) {
        k_txt_fmt<false><<<grid(np, 128), 128, 0, s>>>(d_p, np, fv, slots, lens);
        N2M_COUNT();
        CKL();
    }
    if (nt) {
        k_txt_fmt<true><<<grid(nt, 128), 128, 0, s>>>(d_t, nt, ft, slots + (size_t)(SLOT / 4) * np, lens + np);
        N2M_COUNT();
        CKL();
    }
    CKS(scan_u32(lens, (size_t)nl, lens + nl, sw, s));
    // vertex lines, then mid text, then triangle lines: split the body at the first triangle line
    unsigned body = 0, vbytes = 0;
    CK(cudaMemcpyAsync(&body, lens + nl, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(&vbytes, lens + np, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    const size_t total = head.size() + body + mid.size() + tail.size();
    CKS(w.out.ensure(total + 16));
    Assembler a{w, s};
    CKS(a.text(head));
    unsigned char *o = w.out.as<unsigned char>();
    if (np) {
        k_txt_copy<<<grid(np, 32 * COPY_WARPS), 32 * COPY_WARPS, 0, s>>>(slots, lens, np, o + a.pos);
        N2M_COUNT();
        CKL();
    }
    a.pos += vbytes;
    CKS(a.text(mid));
    if (nt) {
        // offsets of the triangle lines are relative to the start of the body
        k_txt_copy<<<grid(nt, 32 * COPY_WARPS), 32 * COPY_WARPS, 0, s>>>(slots + (size_t)(SLOT / 4) * np, lens + np, nt,
                                                                         o + a.pos - vbytes);
        N2M_COUNT();
        CKL();
    }
    a.pos += body - vbytes;
    CKS(a.text(tail));
    *len = a.pos;
    return N2M_OK;
}

// raw bytes of d_src into a padded scratch buffer (deflate reads 8 bytes past the end), then deflate
n2m_status deflate_from(const void *d_src, size_t n, int container, DevBuf &scratch, WriterWork &w, ScanWork &sw,
                        cudaStream_t s, size_t *clen) {
    CKS(scratch.ensure(n + 16));
    if (n) CK(cudaMemcpyAsync(scratch.p, d_src, n, cudaMemcpyDeviceToDevice, s));
    CK(cudaMemsetAsync(scratch.as<unsigned char>() + n, 0, 16, s));
    CKS(deflate_device(scratch.p, n, container, w.df, sw, s, clen));
    return N2M_OK;
}

std::string gii_array_head(bool tris, int dim0, bool gz) {
    std::string h;
    h += "   <DataArray  ArrayIndexingOrder=\"RowMajorOrder\"\n";
    h += tris ? "               DataType=\"NIFTI_TYPE_INT32\"\n" : "               DataType=\"NIFTI_TYPE_FLOAT32\"\n";
    h += fmt_str("               Dim0=\"%lld\"\n", dim0);
    h += "               Dim1=\"3\"\n";
    h += "               Dimensionality=\"2\"\n";
    h += gz ? "               Encoding=\"GZipBase64Binary\"\n" : "               Encoding=\"Base64Binary\"\n";
    h += "               Endian=\"LittleEndian\"\n";
    h += "               ExternalFileName=\"\"\n";
    h += "               ExternalFileOffset=\"\"\n";
    h += tris ? "               Intent=\"NIFTI_INTENT_TRIANGLE\">\n" : "               Intent=\"NIFTI_INTENT_POINTSET\">\n";
    h += "      <MetaData>\n";
    h += "      </MetaData>\n";
    if (!tris) {
        h += "      <CoordinateSystemTransformMatrix>\n";
        h += "         <DataSpace><![CDATA[NIFTI_XFORM_UNKNOWN]]></DataSpace>\n";
        h += "         <TransformedSpace><![CDATA[NIFTI_XFORM_UNKNOWN]]></TransformedSpace>\n";
        h += "         <MatrixData>1.000000 0.000000 0.000000 0.000000 0.000000 1.000000 0.000000 0.000000 0.000000 "
             "0.000000 1.000000 0.000000 0.000000 0.000000 0.000000 1.000000 </MatrixData>\n";
        h += "      </CoordinateSystemTransformMatrix>\n";
    }
    h += "      <Data>";
    return h;
}

n2m_status encode_gii(const vec3i *d_t, const vec3d *d_p, int nt, int np, bool gz, WriterWork &w, ScanWork &sw,
                      cudaStream_t s, size_t *len) {
    // the two arrays' bytes (zlib-compressed when gz) in w.pack (triangles) and w.pack2 (vertices)
    const size_t tb = (size_t)nt * 12, pb = (size_t)np * 12;
    size_t tlen = tb, plen = pb;
    CKS(w.pack2.ensure(pb + 16));
    if (np) {
        k_pack_pts<<<grid(np, 256), 256, 0, s>>>(d_p, np, w.pack2.as<unsigned char>(), 0);
        N2M_COUNT();
        CKL();
    }
    if (gz) {
        CKS(deflate_from(d_t, tb, N2M_DEFLATE_ZLIB, w.pack, w, sw, s, &tlen));
        CKS(w.pack.ensure(tlen + 16));   // the scratch copy of the triangles is no longer needed
        CK(cudaMemcpyAsync(w.pack.p, w.df.out.p, tlen, cudaMemcpyDeviceToDevice, s));
        CKS(deflate_check(w.df, s));
        CKS(deflate_device(w.pack2.p, pb, N2M_DEFLATE_ZLIB, w.df, sw, s, &plen));
        CKS(w.pack2.ensure(plen + 16));
        CK(cudaMemcpyAsync(w.pack2.p, w.df.out.p, plen, cudaMemcpyDeviceToDevice, s));
        CKS(deflate_check(w.df, s));
    } else {
        CKS(w.pack.ensure(tb + 16));
        if (nt) CK(cudaMemcpyAsync(w.pack.p, d_t, tb, cudaMemcpyDeviceToDevice, s));
    }
    std::string head = "<?xml version=\"1.0\" encoding=\"UTF-8\"?>\n"
                       "<!DOCTYPE GIFTI SYSTEM \"http://www.nitrc.org/frs/download.php/115/gifti.dtd\">\n"
                       "<GIFTI Version=\"1.0\"  NumberOfDataArrays=\"2\">\n"
                       "   <MetaData>\n"
                       "      <MD>\n"
                       "          <Name><![CDATA[nii2mesh-version]]></Name>\n"
                       "          <Value><![CDATA[nii2mesh, 1 Jan 2022]]></Value>\n"
                       "      </MD>\n"
                       "   </MetaData>\n"
                       "   <LabelTable/>\n";
    head += gii_array_head(true, nt, gz);
    const std::string mid = "</Data>\n   </DataArray>\n" + gii_array_head(false, np, gz);
    const std::string tail = "</Data>\n   </DataArray>\n</GIFTI>\n";
    const size_t t64 = 4 * ((tlen + 2) / 3), p64 = 4 * ((plen + 2) / 3);
    CKS(w.out.ensure(head.size() + t64 + mid.size() + p64 + tail.size() + 16));
    Assembler a{w, s};
    unsigned char *o = w.out.as<unsigned char>();
    CKS(a.text(head));
    if (tlen) {
        k_base64<<<grid((long long)(tlen + 2) / 3, 256), 256, 0, s>>>(w.pack.as<unsigned char>(), (long long)tlen, o + a.pos);
        N2M_COUNT();
        CKL();
    }
    a.pos += t64;
    CKS(a.text(mid));
    if (plen) {
        k_base64<<<grid((long long)(plen + 2) / 3, 256), 256, 0, s>>>(w.pack2.as<unsigned char>(), (long long)plen, o + a.pos);
        N2M_COUNT();
        CKL();
    }
    a.pos += p64;
    CKS(a.text(tail));
    *len = a.pos;
    return N2M_OK;
}
}  // namespace

// start of a file name's extension: the last '.' that is not directly after a path separator
// (strip_ext, src/meshify.c:973-982), or the end of the name
const char *file_ext(const char *fnm) {
    const char *end = fnm + strlen(fnm), *dot = end;
    while (dot > fnm && *dot != '.' && *dot != '\\' && *dot != '/') --dot;
    return (dot > fnm && *dot == '.' && dot[-1] != '\\' && dot[-1] != '/') ? dot : end;
}

int mesh_format_of(const char *fnm) {
    // the first format whose name the extension contains wins (src/meshify.c:989-1013)
    const char *ext = file_ext(fnm);
    if (strstr(ext, ".mz3")) return N2M_FMT_MZ3;
    if (strstr(ext, ".gii")) return N2M_FMT_GII;
    if (strstr(ext, ".inflated") || strstr(ext, ".pial")) return N2M_FMT_FREESURFER;
    if (strstr(ext, ".json")) return N2M_FMT_JSON;
    if (strstr(ext, ".off")) return N2M_FMT_OFF;
    if (strstr(ext, ".obj")) return N2M_FMT_OBJ;
    if (strstr(ext, ".ply")) return N2M_FMT_PLY;
    if (strstr(ext, ".stl")) return N2M_FMT_STL;
    if (strstr(ext, ".vtk")) return N2M_FMT_VTK;
    return -1;
}

std::string freesurfer_stamp() {
    const time_t t = time(nullptr);
    struct tm tmv;
    localtime_r(&t, &tmv);
    char s[128] = "";
    strftime(s, sizeof s, "created by niimath on %c\n\n", &tmv);
    return s;
}

n2m_status encode_mesh_device(int format, const vec3i *d_t, const vec3d *d_p, int nt, int np, bool gz, WriterWork &w,
                              ScanWork &sw, cudaStream_t s, const unsigned char **d_out, size_t *len) {
    if (nt < 0 || np < 0 || (nt && !d_t) || (np && !d_p) || format < N2M_FMT_MZ3 || format > N2M_FMT_VTK) {
        n2m_set_error("encode mesh: bad arguments");
        return N2M_ERR_BAD_ARGS;
    }
    const size_t tb = (size_t)nt * 12, pb = (size_t)np * 12;
    *d_out = nullptr;
    switch (format) {
    case N2M_FMT_MZ3: {
        const size_t n = 16 + tb + pb;
        CKS(w.pack.ensure(n + 16));
        unsigned char *d = w.pack.as<unsigned char>();
        unsigned char h[16] = {0x4D, 0x5A, 3, 0};   // "MZ", ATTR 3 (faces + vertices), NFACE, NVERT, NSKIP 0
        for (int i = 0; i < 4; i++) {
            h[4 + i] = (unsigned char)((unsigned)nt >> (8 * i));
            h[8 + i] = (unsigned char)((unsigned)np >> (8 * i));
        }
        CK(cudaMemcpyAsync(d, h, 16, cudaMemcpyHostToDevice, s));
        if (nt) CK(cudaMemcpyAsync(d + 16, d_t, tb, cudaMemcpyDeviceToDevice, s));
        if (np) {
            k_pack_pts<<<grid(np, 256), 256, 0, s>>>(d_p, np, d + 16 + tb, 0);
            N2M_COUNT();
            CKL();
        }
        if (gz) {
            CK(cudaMemsetAsync(d + n, 0, 16, s));
            CKS(deflate_device(d, n, N2M_DEFLATE_GZIP, w.df, sw, s, len));
            CKS(deflate_check(w.df, s));
            *d_out = w.df.out.as<unsigned char>();
        } else {
            *len = n;
            *d_out = d;
        }
        return N2M_OK;
    }
    case N2M_FMT_GII:
        CKS(encode_gii(d_t, d_p, nt, np, gz, w, sw, s, len));
        break;
    case N2M_FMT_JSON:
    case N2M_FMT_OFF:
    case N2M_FMT_OBJ:
        CKS(encode_text(format, d_t, d_p, nt, np, w, sw, s, len));
        break;
    case N2M_FMT_FREESURFER: {
        std::string head("\xFF\xFF\xFE", 3);
        head += freesurfer_stamp();
        unsigned char cnt[8];
        for (int i = 0; i < 4; i++) {
            cnt[i] = (unsigned char)((unsigned)np >> (24 - 8 * i));
            cnt[4 + i] = (unsigned char)((unsigned)nt >> (24 - 8 * i));
        }
        head.append((const char *)cnt, 8);
        CKS(w.out.ensure(head.size() + pb + tb + 16));
        Assembler a{w, s};
        CKS(a.text(head));
        unsigned char *o = w.out.as<unsigned char>();
        if (np) {
            k_pack_pts<<<grid(np, 256), 256, 0, s>>>(d_p, np, o + a.pos, 1);
            N2M_COUNT();
            CKL();
        }
        if (nt) {
            k_pack_tris<<<grid(nt, 256), 256, 0, s>>>(d_t, nt, o + a.pos + pb, TRI_BE12);
            N2M_COUNT();
            CKL();
        }
        *len = a.pos + pb + tb;
        break;
    }
    case N2M_FMT_PLY: {
        std::string head = "ply\nformat binary_little_endian 1.0\ncomment niimath\n";
        head += fmt_str("element vertex %lld\n", np);
        head += "property float x\nproperty float y\nproperty float z\n";
        head += fmt_str("element face %lld\n", nt);
        head += "property list uchar int vertex_indices\nend_header\n";
        CKS(w.out.ensure(head.size() + pb + (size_t)nt * 13 + 16));
        Assembler a{w, s};
        CKS(a.text(head));
        unsigned char *o = w.out.as<unsigned char>();
        if (np) {
            k_pack_pts<<<grid(np, 256), 256, 0, s>>>(d_p, np, o + a.pos, 0);
            N2M_COUNT();
            CKL();
        }
        if (nt) {
            k_pack_tris<<<grid(nt, 256), 256, 0, s>>>(d_t, nt, o + a.pos + pb, TRI_PLY13);
            N2M_COUNT();
            CKL();
        }
        *len = a.pos + pb + (size_t)nt * 13;
        break;
    }
    case N2M_FMT_STL: {
        std::string head(80, '\0');
        unsigned char nf[4];
        for (int i = 0; i < 4; i++) nf[i] = (unsigned char)((unsigned)nt >> (8 * i));
        head.append((const char *)nf, 4);
        CKS(w.out.ensure(head.size() + (size_t)nt * 50 + 16));
        CKS(w.flag.ensure(sizeof(unsigned)));
        CK(cudaMemsetAsync(w.flag.p, 0, sizeof(unsigned), s));
        Assembler a{w, s};
        CKS(a.text(head));
        if (nt) {
            k_pack_stl<<<grid(nt, 256), 256, 0, s>>>(d_t, d_p, nt, np, w.out.as<unsigned char>() + a.pos,
                                                    w.flag.as<unsigned>());
            N2M_COUNT();
            CKL();
        }
        unsigned bad = 0;
        CK(cudaMemcpyAsync(&bad, w.flag.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
        CK(cudaStreamSynchronize(s));
        if (bad) {
            n2m_set_error("save_stl: a triangle refers to a vertex outside [0, %d)", np);
            return N2M_ERR_BAD_ARGS;
        }
        *len = a.pos + (size_t)nt * 50;
        break;
    }
    case N2M_FMT_VTK: {
        std::string head = "# vtk DataFile Version 3.0\nthis file was written using niimath\nBINARY\nDATASET POLYDATA\n";
        head += fmt_str("POINTS %lld float\n", np);
        const std::string mid = fmt_str("POLYGONS %lld %lld\n", nt, 4ll * nt);
        CKS(w.out.ensure(head.size() + pb + mid.size() + (size_t)nt * 16 + 16));
        Assembler a{w, s};
        CKS(a.text(head));
        unsigned char *o = w.out.as<unsigned char>();
        if (np) {
            k_pack_pts<<<grid(np, 256), 256, 0, s>>>(d_p, np, o + a.pos, 1);
            N2M_COUNT();
            CKL();
        }
        a.pos += pb;
        CKS(a.text(mid));
        if (nt) {
            k_pack_tris<<<grid(nt, 256), 256, 0, s>>>(d_t, nt, o + a.pos, TRI_VTK16);
            N2M_COUNT();
            CKL();
        }
        *len = a.pos + (size_t)nt * 16;
        break;
    }
    }
    *d_out = w.out.as<unsigned char>();
    return N2M_OK;
}
