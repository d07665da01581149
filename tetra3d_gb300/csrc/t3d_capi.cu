// t3d_capi.cu -- extern "C" entry points of include/t3d.h (context, scenes,
// frames, CUDA graph replay). Serving lives in t3d_serve.cu.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "t3d_runtime.h"

extern "C" const void* t3d_frame_kernel_ptr();
extern "C" const void* t3d_frame_kernel_mesh_ptr();
extern "C" size_t t3d_frame_smem_bytes(uint32_t tile_tris, uint32_t block_threads);
extern "C" size_t t3d_frame_smem_bytes_mesh(uint32_t tile_tris, uint32_t block_threads, uint32_t mesh_ucap);
extern "C" const void* t3d_phase_kernel_ptr(int mesh, int k);
extern "C" size_t t3d_phase_smem_bytes(int mesh, int k, uint32_t tile_tris, uint32_t block_threads, uint32_t mesh_ucap);

using namespace t3d;

#define CKR(call)                                                                                       \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess) {                                                                        \
            set_err(ctx, "%s failed: %s", #call, cudaGetErrorString(e_));                              \
            return e_ == cudaErrorMemoryAllocation ? T3D_E_OOM : T3D_E_CUDA;                            \
        }                                                                                               \
    } while (0)

namespace t3d {
int configure(t3d_ctx* ctx) {
    ctx->smem_bytes = t3d_frame_smem_bytes(ctx->tile_tris, ctx->block_threads);
    const void* fn = t3d_frame_kernel_ptr();
    CKR(raise_smem_limit(fn, ctx->smem_bytes));
    int per_sm = 0;
    CKR(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, (int)ctx->block_threads, ctx->smem_bytes));
    if (per_sm < 1) {
        set_err(ctx, "frame kernel does not fit on an SM (block %u, smem %zu)", ctx->block_threads, ctx->smem_bytes);
        return T3D_E_INVAL;
    }
    ctx->max_grid = (uint32_t)(per_sm * ctx->num_sms);
    // the meshlet kernel runs two blocks per SM (its register budget); its slot budget per
    // meshlet is the largest (a multiple of 32) that the shared memory of two blocks holds
    ctx->mesh_ucap = 0;
    ctx->smem_mesh = 0;
    ctx->max_grid_mesh = 0;
    int sm_bytes = 0, reserved = 0, block_max = 0;
    CKR(cudaDeviceGetAttribute(&sm_bytes, cudaDevAttrMaxSharedMemoryPerMultiprocessor, ctx->device));
    CKR(cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, ctx->device));
    CKR(cudaDeviceGetAttribute(&block_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device));
    const size_t budget = std::min<size_t>((size_t)block_max, (size_t)(sm_bytes / 2 - reserved));
    // meshlet tiles hold at most 2048 triangles (their rank words keep 11-bit entry numbers)
    uint32_t U = ctx->tile_tris <= 2048 ? std::min<uint32_t>(3 * ctx->tile_tris, 65504u) & ~31u : 0u;
    while (U >= 64 && t3d_frame_smem_bytes_mesh(ctx->tile_tris, ctx->block_threads, U) > budget) U -= 32;
    if (U >= 64) {
        const size_t smem = t3d_frame_smem_bytes_mesh(ctx->tile_tris, ctx->block_threads, U);
        const void* fm = t3d_frame_kernel_mesh_ptr();
        int per = 0;
        if (raise_smem_limit(fm, smem) == cudaSuccess &&
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fm, (int)ctx->block_threads, smem) == cudaSuccess &&
            per >= 1) {
            ctx->mesh_ucap = U;
            ctx->smem_mesh = smem;
            ctx->max_grid_mesh = (uint32_t)(per * ctx->num_sms);
        }
        cudaGetLastError();
    }
    // the one-phase kernels: each with the shared memory of its own phase and its own
    // co-resident blocks (no grid barrier: nothing needs them all resident at once)
    for (int m = 0; m < 2; m++) {
        for (int k = 0; k < 6; k++) {
            ctx->phase_smem[m][k] = 0;
            ctx->phase_grid[m][k] = 0;
            if (m == 1 && !ctx->mesh_ucap) continue;
            const size_t smem = t3d_phase_smem_bytes(m, k, ctx->tile_tris, ctx->block_threads, ctx->mesh_ucap);
            const void* fp = t3d_phase_kernel_ptr(m, k);
            int per = 0;
            if (raise_smem_limit(fp, smem) == cudaSuccess &&
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fp, (int)ctx->block_threads, smem) == cudaSuccess &&
                per >= 1) {
                ctx->phase_smem[m][k] = smem;
                ctx->phase_grid[m][k] = (uint32_t)(per * ctx->num_sms);
            }
            cudaGetLastError();
        }
    }
    return T3D_OK;
}
}  // namespace t3d

static void drop_graph(t3d_ctx* ctx) {
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
    if (ctx->graph) cudaGraphDestroy(ctx->graph);
    ctx->graph_exec = nullptr;
    ctx->graph = nullptr;
}

extern "C" {

int t3d_create(int device, t3d_ctx** out) {
    if (!out) return T3D_E_INVAL;
    *out = nullptr;
    t3d_ctx* ctx = new (std::nothrow) t3d_ctx();
    if (!ctx) return T3D_E_OOM;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || device < 0 || device >= n) {
        delete ctx;
        return T3D_E_CUDA;
    }
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_done, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_upload, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_models, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_readback, cudaEventDisableTiming) != cudaSuccess) {
        delete ctx;
        return T3D_E_CUDA;
    }
    cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device);
    if (!coop) {
        delete ctx;
        return T3D_E_CUDA;
    }
    if (configure(ctx) != T3D_OK || ctx->accum.ensure(ctx, 64) != T3D_OK ||
        cudaMemset(ctx->accum.ptr, 0, ctx->accum.cap) != cudaSuccess) {
        delete ctx;
        return T3D_E_CUDA;
    }
    *out = ctx;
    return T3D_OK;
}

int t3d_destroy(t3d_ctx* ctx) {
    if (!ctx) return T3D_E_INVAL;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->last_stream) cudaStreamSynchronize(ctx->last_stream);
    if (ctx->ev_models) cudaEventSynchronize(ctx->ev_models);
    drop_graph(ctx);
    for (auto& kv : ctx->scenes) kv.second->release();
    ctx->scenes.clear();
    for (DevBuf* b : {&ctx->table_dev, &ctx->ctl, &ctx->preps, &ctx->vcull, &ctx->valt, &ctx->vxyuv, &ctx->vrgba,
                      &ctx->vis_idx, &ctx->vis_depth, &ctx->vis_vloc, &ctx->tile_count, &ctx->tile_wcnt, &ctx->tile_hist,
                      &ctx->chunk_hist, &ctx->seg_minmax, &ctx->seg_count, &ctx->out_xyuv, &ctx->out_rgba, &ctx->out_depth, &ctx->accum, &ctx->inst_lights,
                      &ctx->job_bytes, &ctx->vis_rank, &ctx->vinvw, &ctx->out_invw, &ctx->live_tiles})
        b->release();
    cudaStreamSynchronize(ctx->stream);  // stream-ordered frees of a pooled context have run
    ctx->table_host.release();
    ctx->readback.release();
    if (ctx->ev_done) cudaEventDestroy(ctx->ev_done);
    if (ctx->ev_upload) cudaEventDestroy(ctx->ev_upload);
    if (ctx->ev_models) cudaEventDestroy(ctx->ev_models);
    if (ctx->ev_readback) cudaEventDestroy(ctx->ev_readback);
    ctx->readback2.release();
    t3d_raster_release(ctx);
    ctx->model_host.release();
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return T3D_OK;
}

const char* t3d_last_error(const t3d_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int t3d_set_tuning(t3d_ctx* ctx, uint32_t tile_tris, uint32_t vertex_chunk, uint32_t block_threads) {
    if (!ctx) return T3D_E_INVAL;
    uint32_t T = tile_tris ? tile_tris : ctx->tile_tris;
    uint32_t V = vertex_chunk ? vertex_chunk : ctx->vchunk;
    uint32_t B = block_threads ? block_threads : ctx->block_threads;
    if (T < 256 || T > (uint32_t)kTileMax || (T & (T - 1)) || V < 32 || V > (1u << 20) || (B != 128 && B != 256)) {
        set_err(ctx, "set_tuning: tile %u (256..%d, power of two), chunk %u, block %u (128/256)", T, kTileMax, V, B);
        return T3D_E_INVAL;
    }
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    uint32_t oT = ctx->tile_tris, oV = ctx->vchunk, oB = ctx->block_threads;
    ctx->tile_tris = T;
    ctx->vchunk = V;
    ctx->block_threads = B;
    ctx->tables_ok = false;
    int rc = configure(ctx);
    if (rc) {
        ctx->tile_tris = oT; ctx->vchunk = oV; ctx->block_threads = oB;
        configure(ctx);
        return rc;
    }
    drop_graph(ctx);
    ctx->frame_valid = false;
    return T3D_OK;
}

int t3d_set_meshlets(t3d_ctx* ctx, int enable) {
    if (!ctx) return T3D_E_INVAL;
    cudaSetDevice(ctx->device);
    if (ctx->last_stream) CKR(cudaStreamSynchronize(ctx->last_stream));
    ctx->use_meshlets = enable != 0;
    ctx->tables_ok = false;
    drop_graph(ctx);
    ctx->frame_valid = false;
    return T3D_OK;
}

int t3d_set_split_phases(t3d_ctx* ctx, int mode) {
    if (!ctx || mode < 0 || mode > 1) return T3D_E_INVAL;
    cudaSetDevice(ctx->device);
    if (ctx->last_stream) CKR(cudaStreamSynchronize(ctx->last_stream));
    ctx->split_phases = mode != 0;
    drop_graph(ctx);
    return T3D_OK;
}

int t3d_set_wait_limit(t3d_ctx* ctx, uint32_t polls) {
    if (!ctx) return T3D_E_INVAL;
    cudaSetDevice(ctx->device);
    if (ctx->last_stream) CKR(cudaStreamSynchronize(ctx->last_stream));
    ctx->spin_limit = polls;
    ctx->params.spin_limit = polls;
    ctx->tables_ok = false;  // the limit travels in the launch parameters
    drop_graph(ctx);
    return T3D_OK;
}

int t3d_scene_upload(t3d_ctx* ctx, const t3d_scene_desc* desc, uint32_t* scene_out) {
    if (!ctx) return T3D_E_INVAL;
    cudaSetDevice(ctx->device);
    return scene_upload(ctx, desc, scene_out);
}

int t3d_scene_release(t3d_ctx* ctx, uint32_t scene) {
    if (!ctx) return T3D_E_INVAL;
    auto it = ctx->scenes.find(scene);
    if (it == ctx->scenes.end()) return T3D_E_NOTFOUND;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->last_stream) cudaStreamSynchronize(ctx->last_stream);
    drop_graph(ctx);
    ctx->frame_valid = false;
    it->second->release();
    ctx->scenes.erase(it);
    return T3D_OK;
}

int t3d_scene_set_models(t3d_ctx* ctx, uint32_t scene, uint32_t first, const t3d_model_desc* models, uint32_t n) {
    if (!ctx || (n && !models)) return T3D_E_INVAL;
    auto it = ctx->scenes.find(scene);
    if (it == ctx->scenes.end()) return T3D_E_NOTFOUND;
    Scene* sc = it->second.get();
    if ((uint64_t)first + n > sc->models.size()) {
        set_err(ctx, "set_models: range [%u, %u) beyond %zu models", first, first + n, sc->models.size());
        return T3D_E_INVAL;
    }
    for (uint32_t i = 0; i < n; i++) {
        if (models[i].mesh >= sc->meshes.size() || models[i].light_list >= (int32_t)sc->lists.size()) {
            set_err(ctx, "set_models: model %u has a bad mesh or light list", first + i);
            return T3D_E_INVAL;
        }
        if (models[i].batched) {
            const uint32_t o = models[i].batch_owner;
            const uint32_t omesh = (o >= first && o < first + n) ? models[o - first].mesh
                                   : (o < sc->models.size() ? sc->models[o].d.mesh : 0xFFFFFFFFu);
            if (o >= sc->models.size() || o == first + i || omesh >= sc->meshes.size() ||
                models[i].batch_part >= sc->meshes[omesh].parts.size()) {
                set_err(ctx, "set_models: model %u: batch owner %u or its part %u out of range", first + i, o,
                        models[i].batch_part);
                return T3D_E_INVAL;
            }
        }
        const SceneMesh& me = sc->meshes[models[i].mesh];
        if (models[i].skinned && (!me.skin || me.subdiv || (uint64_t)models[i].bone_first + me.max_joint >= sc->num_bones)) {
            set_err(ctx, "set_models: skinned model %u without joints or with bones beyond the scene's %u", first + i,
                    sc->num_bones);
            return T3D_E_INVAL;
        }
    }
    cudaSetDevice(ctx->device);
    // no host wait: the copy is queued behind the frames already issued (scene_write_models)
    return scene_write_models(ctx, sc, first, models, n);
}

int t3d_scene_get_transforms(t3d_ctx* ctx, uint32_t scene, float* out, uint32_t n) {
    if (!ctx || !out) return T3D_E_INVAL;
    auto it = ctx->scenes.find(scene);
    if (it == ctx->scenes.end()) return T3D_E_NOTFOUND;
    Scene* sc = it->second.get();
    n = std::min<uint32_t>(n, (uint32_t)sc->models.size());
    cudaSetDevice(ctx->device);
    if (ctx->last_stream) CKR(cudaStreamSynchronize(ctx->last_stream));
    if (ctx->ev_models) CKR(cudaEventSynchronize(ctx->ev_models));
    std::vector<DevModel> dm(n);
    if (n) CKR(cudaMemcpy(dm.data(), sc->dmodels.ptr, sizeof(DevModel) * n, cudaMemcpyDeviceToHost));
    for (uint32_t i = 0; i < n; i++) {
        const DevModel& m = dm[i];
        if (m.flags & MOD_TRS) {
            m4 M = trs(mk3(m.position[0], m.position[1], m.position[2]), mk3(m.scale[0], m.scale[1], m.scale[2]),
                       load16(m.rotation));
            store16(M, out + 16 * (size_t)i);
        } else {
            memcpy(out + 16 * (size_t)i, m.transform, 64);
        }
    }
    return T3D_OK;
}

int t3d_scene_set_bones(t3d_ctx* ctx, uint32_t scene, uint32_t first, const float* influences, uint32_t n) {
    if (!ctx || (n && !influences)) return T3D_E_INVAL;
    auto it = ctx->scenes.find(scene);
    if (it == ctx->scenes.end()) return T3D_E_NOTFOUND;
    Scene* sc = it->second.get();
    if ((uint64_t)first + n > sc->num_bones) {
        set_err(ctx, "set_bones: range [%u, %u) beyond %u bones", first, first + n, sc->num_bones);
        return T3D_E_INVAL;
    }
    cudaSetDevice(ctx->device);
    if (ctx->last_stream) CKR(cudaStreamSynchronize(ctx->last_stream));
    if (n) CKR(cudaMemcpy((char*)sc->bones.ptr + 64ull * first, influences, 64ull * n, cudaMemcpyHostToDevice));
    return T3D_OK;
}

int t3d_scene_set_shape_weights(t3d_ctx* ctx, uint32_t scene, uint32_t mesh, const float* weights, uint32_t n) {
    if (!ctx || (n && !weights)) return T3D_E_INVAL;
    auto it = ctx->scenes.find(scene);
    if (it == ctx->scenes.end()) return T3D_E_NOTFOUND;
    Scene* sc = it->second.get();
    if (mesh >= sc->meshes.size() || n != sc->meshes[mesh].nkeys) {
        set_err(ctx, "set_shape_weights: mesh %u out of range or %u weights for its shape keys", mesh, n);
        return T3D_E_INVAL;
    }
    cudaSetDevice(ctx->device);
    if (ctx->last_stream) CKR(cudaStreamSynchronize(ctx->last_stream));
    if (n) {
        CKR(cudaMemcpy((float*)sc->shape_w.ptr + sc->meshes[mesh].weight_first, weights, 4ull * n,
                       cudaMemcpyHostToDevice));
        int rc;
        if ((rc = bake_shapes(ctx, sc, mesh))) return rc;  // the mesh's keyed streams for the new weights
        if ((rc = fill_keyed_meshlets(ctx, sc, mesh))) return rc;  // and its meshlets' vertex data
        CKR(cudaStreamSynchronize(ctx->stream));
    }
    return T3D_OK;
}

int t3d_scene_set_lights(t3d_ctx* ctx, uint32_t scene, uint32_t first, const t3d_light_desc* lights, uint32_t n) {
    if (!ctx || (n && !lights)) return T3D_E_INVAL;
    auto it = ctx->scenes.find(scene);
    if (it == ctx->scenes.end()) return T3D_E_NOTFOUND;
    Scene* sc = it->second.get();
    if ((uint64_t)first + n > sc->lights.size()) {
        set_err(ctx, "set_lights: range [%u, %u) beyond %zu lights", first, first + n, sc->lights.size());
        return T3D_E_INVAL;
    }
    for (uint32_t i = 0; i < n; i++) {
        const t3d_light_desc& l = lights[i];
        if (l.type < 0 || l.type > 3) {
            set_err(ctx, "set_lights: light %u has bad type %d", first + i, l.type);
            return T3D_E_INVAL;
        }
        if (l.type == T3D_LIGHT_VOLUME && sc->light_nested[first + i]) {
            set_err(ctx, "set_lights: light %u is used by light-volume cells and cannot become a volume", first + i);
            return T3D_E_INVAL;
        }
        if (l.type == T3D_LIGHT_VOLUME) {
            const uint64_t cells = (uint64_t)std::max(0, l.cell_count[0]) * std::max(0, l.cell_count[1]) *
                                   std::max(0, l.cell_count[2]);
            if ((uint64_t)l.cell_first + cells > sc->num_cells) {
                set_err(ctx, "set_lights: light %u: volume cells out of range", first + i);
                return T3D_E_INVAL;
            }
        }
    }
    cudaSetDevice(ctx->device);
    // the light tables of frames in flight are already on the device; the next
    // render builds new ones, so only a captured graph (which keeps its tables) goes
    if (ctx->last_stream) CKR(cudaStreamSynchronize(ctx->last_stream));
    drop_graph(ctx);
    for (uint32_t i = 0; i < n; i++) {
        sc->lights[first + i] = lights[i];
        const t3d_light_desc& l = lights[i];
        sc->light_uses[first + i] = 0;  // a volume's cells keep their use lists; its cell range may move
        if (l.type == T3D_LIGHT_VOLUME) {
            const uint64_t cells = (uint64_t)std::max(0, l.cell_count[0]) * std::max(0, l.cell_count[1]) *
                                   std::max(0, l.cell_count[2]);
            sc->light_uses[first + i] = sc->cell_uses_between(l.cell_first, l.cell_first + cells);
        }
    }
    sc->struct_ver = next_version();
    return T3D_OK;
}

int t3d_scene_bytes(t3d_ctx* ctx, uint32_t scene, uint64_t* bytes_out) {
    if (!ctx || !bytes_out) return T3D_E_INVAL;
    auto it = ctx->scenes.find(scene);
    if (it == ctx->scenes.end()) return T3D_E_NOTFOUND;
    *bytes_out = it->second->device_bytes();
    return T3D_OK;
}

int t3d_render_jobs(t3d_ctx* ctx, const t3d_job_desc* jobs, uint32_t num_jobs, int mode, int animate, void* stream) {
    if (!ctx || (num_jobs && !jobs) || (mode != T3D_MODE_PLAIN && mode != T3D_MODE_BATCHED)) return T3D_E_INVAL;
    if (animate) {
        for (uint32_t a = 0; a < num_jobs; a++)
            for (uint32_t b = a + 1; b < num_jobs; b++)
                if (jobs[a].scene == jobs[b].scene) {
                    set_err(ctx, "animate: scene %u appears in more than one job", jobs[a].scene);
                    return T3D_E_INVAL;
                }
    }
    cudaSetDevice(ctx->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    if (ctx->last_stream && ctx->last_stream != st) CKR(cudaStreamSynchronize(ctx->last_stream));
    {  // model writes to the scenes come first (a serving slot's scenes belong to its parent)
        t3d_ctx* owner = ctx->scene_owner ? ctx->scene_owner : ctx;
        if (owner->ev_models) CKR(cudaStreamWaitEvent(st, owner->ev_models, 0));
    }
    ctx->frame_valid = false;
    // The launch tables depend on the jobs, the tuning and the scenes' structure,
    // and on model transforms only through the draw order of transparent pairs (or
    // of all pairs when depth rendering is off). A render that changes none of
    // these reuses the tables already in the device arena.
    std::vector<unsigned char> sig;
    std::vector<uint64_t> mvers;
    auto put = [&sig](const void* p, size_t n) { sig.insert(sig.end(), (const unsigned char*)p, (const unsigned char*)p + n); };
    const uint32_t knobs[6] = {(uint32_t)mode, (uint32_t)animate, ctx->tile_tris, ctx->vchunk, ctx->block_threads, ctx->max_grid};
    put(knobs, sizeof knobs);
    if (num_jobs) put(jobs, sizeof(t3d_job_desc) * num_jobs);
    bool known = true;
    for (uint32_t j = 0; j < num_jobs; j++) {
        auto it = ctx->scene_map().find(jobs[j].scene);
        if (it == ctx->scene_map().end()) { known = false; break; }
        put(&it->second->struct_ver, sizeof(uint64_t));
        mvers.push_back(it->second->model_ver);
    }
    const bool reuse = known && !animate && ctx->tables_ok && sig == ctx->table_sig &&
                       (!ctx->order_dep || mvers == ctx->table_model_vers);
    int rc;
    if (!reuse) {
        drop_graph(ctx);  // a captured graph reads the arena that is rewritten now
        if ((rc = build_frame(ctx, jobs, num_jobs, animate))) return rc;
        // The table arena is reused: the previous frame must have consumed it.
        if ((rc = upload_frame(ctx, st))) return rc;
        ctx->table_sig.swap(sig);
        ctx->table_model_vers.swap(mvers);
        ctx->tables_ok = true;
    } else {
        ctx->last_h2d = 0;
    }
    if ((rc = launch_frame(ctx, mode, st))) return rc;
    ctx->last_stream = st;
    ctx->frame_pending = true;
    return T3D_OK;
}

int t3d_render(t3d_ctx* ctx, uint32_t scene, const t3d_camera_desc* cam, int mode, int animate, void* stream) {
    if (!ctx || !cam) return T3D_E_INVAL;
    t3d_job_desc job;
    memset(&job, 0, sizeof job);
    job.scene = scene;
    job.light_mask[0] = job.light_mask[1] = ~0ull;
    job.camera = *cam;
    return t3d_render_jobs(ctx, &job, 1, mode, animate, stream);
}

int t3d_frame_sync(t3d_ctx* ctx, t3d_stats* stats_out) {
    if (!ctx) return T3D_E_INVAL;
    cudaSetDevice(ctx->device);
    if (!ctx->frame_pending && !ctx->frame_valid) {
        set_err(ctx, "frame_sync: no frame rendered");
        return T3D_E_INVAL;
    }
    cudaStream_t st = ctx->last_stream ? ctx->last_stream : ctx->stream;
    FrameTables& F = ctx->tables;
    const size_t nseg = F.segs.size();
    // one read-back: per-pair counts, the launch control blocks and (serving slots) the
    // per-job algorithmic bytes
    const size_t njb = (ctx->want_job_bytes && ctx->params.job_bytes) ? F.jobs.size() : 0;
    const size_t ctl_off = (4 * nseg + 63) & ~(size_t)63;
    const size_t jb_off = ctl_off + sizeof(Ctl) * ctx->nctl;
    const size_t rb = jb_off + 8 * njb + 64;
    if (ctx->readback.ensure(rb)) { set_err(ctx, "pinned readback alloc failed"); return T3D_E_OOM; }
    uint32_t* counts = (uint32_t*)ctx->readback.ptr;
    Ctl* ctls = (Ctl*)((char*)ctx->readback.ptr + ctl_off);
    unsigned long long* jbh = (unsigned long long*)((char*)ctx->readback.ptr + jb_off);
    if (nseg) CKR(cudaMemcpyAsync(counts, ctx->seg_count.ptr, 4 * nseg, cudaMemcpyDeviceToHost, st));
    if (ctx->nctl) CKR(cudaMemcpyAsync(ctls, ctx->ctl.ptr, sizeof(Ctl) * ctx->nctl, cudaMemcpyDeviceToHost, st));
    if (njb) CKR(cudaMemcpyAsync(jbh, ctx->job_bytes.ptr, 8 * njb, cudaMemcpyDeviceToHost, st));
    CKR(cudaStreamSynchronize(st));
    ctx->job_bytes_host.assign(jbh, jbh + njb);
    ctx->frame_pending = false;
    t3d_stats s;
    memset(&s, 0, sizeof s);
    for (uint32_t i = 0; i < ctx->nctl; i++) {
        if (ctls[i].err) {
            set_err(ctx, "frame kernel reported error %d (launch %u)", ctls[i].err, i);
            ctx->frame_valid = false;
            return (ctls[i].err == ERR_BARRIER_TIMEOUT || ctls[i].err == ERR_COPY_TIMEOUT) ? T3D_E_TIMEOUT : T3D_E_CUDA;
        }
        s.algorithmic_bytes += ctls[i].bytes;
        s.culled_models += ctls[i].culled;
    }
    for (size_t k = 0; k < nseg; k++) {
        F.seg_info[k].count = counts[k];
        s.visible_tris += counts[k];
        s.total_tris += F.seg_info[k].capacity;
        if (counts[k]) s.drawn_parts++;
    }
    s.total_parts = (uint32_t)nseg;
    s.algorithmic_bytes += 108ull * s.visible_tris;
    s.launches = ctx->launches;
    size_t scratch = 0;
    for (DevBuf* b : {&ctx->table_dev, &ctx->ctl, &ctx->preps, &ctx->vcull, &ctx->valt, &ctx->vxyuv, &ctx->vrgba,
                      &ctx->vis_idx, &ctx->vis_depth, &ctx->vis_vloc, &ctx->tile_count, &ctx->tile_wcnt, &ctx->tile_hist,
                      &ctx->chunk_hist, &ctx->seg_minmax, &ctx->seg_count, &ctx->inst_lights, &ctx->vis_rank, &ctx->vinvw})
        scratch += b->cap;
    s.scratch_bytes = scratch;
    s.h2d_bytes = ctx->last_h2d;
    if (ctx->nctl == 1) {
        const Ctl& c = ctls[0];
        unsigned long long prev = c.t_end[7];
        const int order[6] = {0, 6, 1, 2, 3, 4};  // prep, vertex, triangles, hist, scan, rank + emit
        for (int i = 0; i < 6; i++) {
            const unsigned long long t = c.t_end[order[i]];
            if (t >= prev && prev) {
                s.phase_us[i] = (double)(t - prev) / 1e3;
                prev = t;
            }
            // order[i] is the timer slot of phase i (prep, vertex, triangles, hist, scan, rank + emit)
            const uint32_t g = ctx->phase_grid_used[i];
            s.phase_busy[i] = g ? (double)c.busy[order[i]] / 1e3 / g : 0.0;
        }
    }
    s.d2h_bytes = 4 * nseg + sizeof(Ctl) * ctx->nctl + 8 * njb;
    ctx->stats = s;
    ctx->frame_valid = true;
    if (stats_out) *stats_out = s;
    return T3D_OK;
}

int t3d_frame_readback(t3d_ctx* ctx) {
    if (!ctx) return T3D_E_INVAL;
    if (!ctx->frame_pending && !ctx->frame_valid) {
        set_err(ctx, "frame_readback: no frame rendered");
        return T3D_E_INVAL;
    }
    if (ctx->rb2_pending) {
        set_err(ctx, "frame_readback: the previous read-back was not collected");
        return T3D_E_INVAL;
    }
    cudaSetDevice(ctx->device);
    cudaStream_t st = ctx->last_stream ? ctx->last_stream : ctx->stream;
    FrameTables& F = ctx->tables;
    const size_t nseg = F.segs.size();
    const size_t ctl_off = (4 * nseg + 63) & ~(size_t)63;
    if (ctx->readback2.ensure(ctl_off + sizeof(Ctl) * ctx->nctl + 64)) {
        set_err(ctx, "pinned readback alloc failed");
        return T3D_E_OOM;
    }
    if (nseg) CKR(cudaMemcpyAsync(ctx->readback2.ptr, ctx->seg_count.ptr, 4 * nseg, cudaMemcpyDeviceToHost, st));
    if (ctx->nctl)
        CKR(cudaMemcpyAsync((char*)ctx->readback2.ptr + ctl_off, ctx->ctl.ptr, sizeof(Ctl) * ctx->nctl,
                            cudaMemcpyDeviceToHost, st));
    CKR(cudaEventRecord(ctx->ev_readback, st));
    uint64_t total = 0;
    for (const auto& si : F.seg_info) total += si.capacity;
    ctx->rb2_nseg = nseg;
    ctx->rb2_nctl = ctx->nctl;
    ctx->rb2_launches = ctx->launches;
    ctx->rb2_total = total;
    ctx->rb2_h2d = ctx->last_h2d;
    ctx->rb2_pending = true;
    return T3D_OK;
}

int t3d_frame_collect(t3d_ctx* ctx, t3d_stats* stats_out) {
    if (!ctx) return T3D_E_INVAL;
    if (!ctx->rb2_pending) {
        set_err(ctx, "frame_collect: no read-back in flight");
        return T3D_E_INVAL;
    }
    cudaSetDevice(ctx->device);
    ctx->rb2_pending = false;
    CKR(cudaEventSynchronize(ctx->ev_readback));
    const uint32_t* counts = (const uint32_t*)ctx->readback2.ptr;
    const Ctl* ctls = (const Ctl*)((const char*)ctx->readback2.ptr + ((4 * ctx->rb2_nseg + 63) & ~(size_t)63));
    t3d_stats s;
    memset(&s, 0, sizeof s);
    for (uint32_t i = 0; i < ctx->rb2_nctl; i++) {
        if (ctls[i].err) {
            set_err(ctx, "frame kernel reported error %d (launch %u)", ctls[i].err, i);
            return (ctls[i].err == ERR_BARRIER_TIMEOUT || ctls[i].err == ERR_COPY_TIMEOUT) ? T3D_E_TIMEOUT : T3D_E_CUDA;
        }
        s.algorithmic_bytes += ctls[i].bytes;
        s.culled_models += ctls[i].culled;
    }
    for (size_t k = 0; k < ctx->rb2_nseg; k++) {
        s.visible_tris += counts[k];
        if (counts[k]) s.drawn_parts++;
    }
    s.total_tris = ctx->rb2_total;
    s.total_parts = (uint32_t)ctx->rb2_nseg;
    s.algorithmic_bytes += 108ull * s.visible_tris;
    s.launches = ctx->rb2_launches;
    s.h2d_bytes = ctx->rb2_h2d;
    s.d2h_bytes = 4 * ctx->rb2_nseg + sizeof(Ctl) * ctx->rb2_nctl;
    if (stats_out) *stats_out = s;
    return T3D_OK;
}

int t3d_frame_counters(t3d_ctx* ctx, uint64_t* visible_total, uint64_t* model_bytes_total) {
    if (!ctx) return T3D_E_INVAL;
    cudaSetDevice(ctx->device);
    unsigned long long h[2] = {0, 0};
    if (ctx->last_stream) CKR(cudaStreamSynchronize(ctx->last_stream));
    CKR(cudaMemcpy(h, ctx->accum.ptr, sizeof h, cudaMemcpyDeviceToHost));
    if (visible_total) *visible_total = h[0];
    if (model_bytes_total) *model_bytes_total = h[1];
    return T3D_OK;
}

int t3d_frame_view_get(t3d_ctx* ctx, t3d_frame_view* v) {
    if (!ctx || !v) return T3D_E_INVAL;
    v->xyuv = (float*)ctx->out_xyuv.ptr;
    v->rgba = (float*)ctx->out_rgba.ptr;
    v->depth = (float*)ctx->out_depth.ptr;
    v->seg_base = nullptr;
    v->seg_count = (uint32_t*)ctx->seg_count.ptr;
    v->num_segments = (uint32_t)ctx->tables.segs.size();
    v->reserved = 0;
    v->capacity_tris = ctx->tables.nslots;
    return T3D_OK;
}

int t3d_frame_segments(t3d_ctx* ctx, t3d_segment_info* segs, uint32_t max_segs, uint32_t* num_out) {
    if (!ctx || !num_out) return T3D_E_INVAL;
    const auto& info = ctx->tables.seg_info;
    *num_out = (uint32_t)info.size();
    if (segs) memcpy(segs, info.data(), sizeof(t3d_segment_info) * std::min<size_t>(max_segs, info.size()));
    return T3D_OK;
}

int t3d_frame_download(t3d_ctx* ctx, float* xyuv, float* rgba, float* depth, uint64_t max_tris, uint64_t* tris_out) {
    if (!ctx) return T3D_E_INVAL;
    if (!ctx->frame_valid) {
        set_err(ctx, "frame_download: call t3d_frame_sync first");
        return T3D_E_INVAL;
    }
    cudaSetDevice(ctx->device);
    uint64_t n = 0;
    for (const auto& si : ctx->tables.seg_info) {
        if (!si.count) continue;
        if (n + si.count > max_tris) {
            set_err(ctx, "frame_download: %llu triangles do not fit %llu", (unsigned long long)(n + si.count),
                    (unsigned long long)max_tris);
            return T3D_E_INVAL;
        }
        if (xyuv) CKR(cudaMemcpy(xyuv + 12 * n, (char*)ctx->out_xyuv.ptr + 48ull * si.base, 48ull * si.count, cudaMemcpyDeviceToHost));
        if (rgba) CKR(cudaMemcpy(rgba + 12 * n, (char*)ctx->out_rgba.ptr + 48ull * si.base, 48ull * si.count, cudaMemcpyDeviceToHost));
        if (depth) CKR(cudaMemcpy(depth + 3 * n, (char*)ctx->out_depth.ptr + 12ull * si.base, 12ull * si.count, cudaMemcpyDeviceToHost));
        n += si.count;
    }
    if (tris_out) *tris_out = n;
    return T3D_OK;
}

int t3d_frame_download_custom0(t3d_ctx* ctx, float* custom0, uint64_t max_tris, uint64_t* tris_out) {
    if (!ctx || !custom0) return T3D_E_INVAL;
    if (!ctx->frame_valid) {
        set_err(ctx, "frame_download_custom0: call t3d_frame_sync first");
        return T3D_E_INVAL;
    }
    if (!ctx->tables.any_pcorrect) {
        set_err(ctx, "frame_download_custom0: no job of the last frame uses perspective-corrected texture mapping");
        return T3D_E_INVAL;
    }
    cudaSetDevice(ctx->device);
    uint64_t n = 0;
    for (size_t k = 0; k < ctx->tables.seg_info.size(); k++) {
        const auto& si = ctx->tables.seg_info[k];
        if (!si.count) continue;
        if (n + si.count > max_tris) {
            set_err(ctx, "frame_download_custom0: %llu triangles do not fit %llu", (unsigned long long)(n + si.count),
                    (unsigned long long)max_tris);
            return T3D_E_INVAL;
        }
        if (ctx->tables.segs[k].flags & SEG_PCORRECT)
            CKR(cudaMemcpy(custom0 + 3 * n, (char*)ctx->out_invw.ptr + 12ull * si.base, 12ull * si.count,
                           cudaMemcpyDeviceToHost));
        else
            memset(custom0 + 3 * n, 0, 12ull * si.count);
        n += si.count;
    }
    if (tris_out) *tris_out = n;
    return T3D_OK;
}

int t3d_graph_capture(t3d_ctx* ctx, uint32_t scene, const t3d_camera_desc* cam, int animate) {
    if (!ctx || !cam) return T3D_E_INVAL;
    cudaSetDevice(ctx->device);
    drop_graph(ctx);
    t3d_job_desc job;
    memset(&job, 0, sizeof job);
    job.scene = scene;
    job.light_mask[0] = job.light_mask[1] = ~0ull;
    job.camera = *cam;
    if (ctx->last_stream) CKR(cudaStreamSynchronize(ctx->last_stream));
    if (ctx->ev_models) CKR(cudaEventSynchronize(ctx->ev_models));
    ctx->tables_ok = false;  // the arena now holds the captured frame's tables
    int rc = build_frame(ctx, &job, 1, animate);
    if (rc) return rc;
    if ((rc = upload_frame(ctx, ctx->stream))) return rc;
    ctx->tables_ok = false;
    if ((rc = ctx->ctl.ensure(ctx, sizeof(Ctl)))) return rc;  // no allocation may happen while capturing
    CKR(cudaStreamSynchronize(ctx->stream));
    CKR(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    rc = launch_frame(ctx, T3D_MODE_BATCHED, ctx->stream);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) {
        set_err(ctx, "graph capture: %s", cudaGetErrorString(e));
        return T3D_E_CUDA;
    }
    ctx->graph = g;
    e = cudaGraphInstantiate(&ctx->graph_exec, g, 0);
    if (e != cudaSuccess) {
        set_err(ctx, "graph instantiate: %s", cudaGetErrorString(e));
        drop_graph(ctx);
        return T3D_E_CUDA;
    }
    ctx->frame_valid = false;
    ctx->frame_pending = false;
    return T3D_OK;
}

int t3d_graph_replay(t3d_ctx* ctx, uint32_t frames, void* stream) {
    if (!ctx || !ctx->graph_exec) {
        if (ctx) set_err(ctx, "graph_replay: no captured graph");
        return T3D_E_INVAL;
    }
    cudaSetDevice(ctx->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
    if (ctx->ev_models) CKR(cudaStreamWaitEvent(st, ctx->ev_models, 0));
    for (uint32_t f = 0; f < frames; f++) CKR(cudaGraphLaunch(ctx->graph_exec, st));
    ctx->last_stream = st;
    ctx->frame_pending = true;
    return T3D_OK;
}

}  // extern "C"
