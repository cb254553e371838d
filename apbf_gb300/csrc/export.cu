// export.cu -- save_particle_info::apply (source/save_particle_info.cpp:22-125): the
// particle state as the reference's text files, for offline comparison with a run
// of the reference.  Host code: the lists are copied to the host, the files are
// written with the reference's formatting (std::ostream defaults, ';' separated
// value files and data.csv sorted by distance to a centre point).  The reference
// sorts data.csv with std::sort, whose order of equal distances is unspecified;
// here it is stable (equal distances keep the particle order).
#include <algorithm>
#include <cmath>
#include <filesystem>
#include <fstream>
#include <numeric>
#include <vector>

#include "apbf_internal.cuh"

using namespace apbf;

extern "C" apbf_status apbf_save_particle_info(apbf_ctx *ctx, const char *folder, const float center[3], void *stream) {
    if (!ctx || !folder || !center) return APBF_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    cudaStream_t s = (cudaStream_t)stream;
    uint32_t n = 0;
    APBF_CUDA(cudaMemcpyAsync(&n, ctx->d_len + kLenParticles, sizeof(n), cudaMemcpyDeviceToHost, s));
    APBF_CUDA(cudaStreamSynchronize(s));
    const FluidBufs &f = ctx->fl[ctx->fcur];
    std::vector<int4> pos(n);
    std::vector<float> radius(n), kw(n), target(n), im(n);
    std::vector<uint32_t> bd(n), cnt(n);
    if (n) {
        APBF_CUDA(cudaMemcpyAsync(pos.data(), f.pos, n * sizeof(int4), cudaMemcpyDeviceToHost, s));
        APBF_CUDA(cudaMemcpyAsync(radius.data(), f.radius, n * 4, cudaMemcpyDeviceToHost, s));
        APBF_CUDA(cudaMemcpyAsync(kw.data(), f.kernel_width, n * 4, cudaMemcpyDeviceToHost, s));
        APBF_CUDA(cudaMemcpyAsync(target.data(), f.target_radius, n * 4, cudaMemcpyDeviceToHost, s));
        APBF_CUDA(cudaMemcpyAsync(im.data(), f.inv_mass, n * 4, cudaMemcpyDeviceToHost, s));
        APBF_CUDA(cudaMemcpyAsync(bd.data(), f.boundary_distance, n * 4, cudaMemcpyDeviceToHost, s));
        // neighbour count per particle = pairs (i, j) of the last search (nbrCount[pair.x]++)
        APBF_CUDA(cudaMemcpyAsync(cnt.data(), ctx->nb_count, n * 4, cudaMemcpyDeviceToHost, s));
        APBF_CUDA(cudaStreamSynchronize(s));
    }
    std::vector<float> cdist(n), bdist(n);
    std::vector<float> px(n), py(n), pz(n);
    for (uint32_t i = 0; i < n; ++i) {
        px[i] = (float)pos[i].x / 262144.0f;
        py[i] = (float)pos[i].y / 262144.0f;
        pz[i] = (float)pos[i].z / 262144.0f;
        bdist[i] = (float)bd[i] / 262144.0f;
        const float dx = px[i] - center[0], dy = py[i] - center[1], dz = pz[i] - center[2];
        cdist[i] = std::sqrt(dx * dx + dy * dy + dz * dz);
    }
    std::error_code ec;
    std::filesystem::create_directories(folder, ec);
    if (ec) {
        set_error(std::string("apbf_save_particle_info: cannot create ") + folder);
        return APBF_ERR_INVALID_ARG;
    }
    const std::string dir(folder);
    auto write_list = [&](const char *name, auto &&value) {
        std::ofstream out(dir + "/" + name);
        for (uint32_t i = 0; i < n; ++i) out << value(i) << ";";
        return (bool)out;
    };
    bool ok = write_list("centerDist.txt", [&](uint32_t i) { return cdist[i]; }) &&
              write_list("radius.txt", [&](uint32_t i) { return radius[i]; }) &&
              write_list("neighborCount.txt", [&](uint32_t i) { return cnt[i]; }) &&
              write_list("kernelWidth.txt", [&](uint32_t i) { return kw[i]; }) &&
              write_list("targetRadius.txt", [&](uint32_t i) { return target[i]; }) &&
              write_list("boundaryDistance.txt", [&](uint32_t i) { return bdist[i]; });
    std::vector<uint32_t> order(n);
    std::iota(order.begin(), order.end(), 0u);
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return cdist[a] < cdist[b]; });
    {
        std::ofstream out(dir + "/data.csv");
        out << "center distance,boundary distance,kernel width,neighbor count,radius,target radius,inverse mass,x,y,z"
            << std::endl;
        for (uint32_t k = 0; k < n; ++k) {
            const uint32_t i = order[k];
            out << cdist[i] << "," << bdist[i] << "," << kw[i] << "," << cnt[i] << "," << radius[i] << ","
                << target[i] << "," << im[i] << "," << px[i] << "," << py[i] << "," << pz[i] << std::endl;
        }
        ok = ok && (bool)out;
    }
    if (!ok) {
        set_error("apbf_save_particle_info: write failed in " + dir);
        return APBF_ERR_INVALID_ARG;
    }
    return APBF_OK;
}
