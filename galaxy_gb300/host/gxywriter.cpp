// gxywriter.cpp -- Galaxy's batch renderer (src/apps/gxywriter.cpp:61-219)
// on the device path: reads a state file, renders every camera x
// visualization, and writes each image; the C++ host classes of
// galaxy_host.hpp over libgxy_gpu.so.
//
//   gxywriter [-s W H] [-p PX PY PZ] [-o PREFIX] [-d DEVICE] [-R PARTITION] [-n] STATE
//
// -s overrides the image size, -p sets the brick grid (Galaxy's
// global_partitions), -o the output prefix: PREFIX_NNNNN.rgba holds each
// image as height x width x 4 float32 (y = 0 the bottom row).  -R also
// checks the RayList path on that partition: camera rays, TraceRays::Trace,
// then the secondaries traced again, with the counts printed.  One JSON
// line per rendering on stdout.  -n renders nothing and needs no GPU: it
// prints what the state file became -- each rendering's camera, resolved
// lighting and transfer-function tables (hexadecimal floats).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "galaxy_host.hpp"

using namespace gxyhost;

static int usage() {
    fprintf(stderr, "usage: gxywriter [-s W H] [-p PX PY PZ] [-o PREFIX] [-d DEVICE] [-R PARTITION] [-n] STATE\n");
    return 2;
}

static void hexfloats(const float *v, int n) {
    printf("[");
    for (int k = 0; k < n; k++) printf("%s\"%a\"", k ? ", " : "", (double)v[k]);
    printf("]");
}

// -n: the parsed scene, without a device
static void describe(const Rendering &r) {
    gxy_camera c = r.camera.c();
    gxy_lighting in = r.vis->lighting.c(), L;
    check(gxy_resolve_lights(&in, &c, &L));
    printf("{\"camera\": {\"eye\": ");
    hexfloats(c.eye, 3);
    printf(", \"dir\": ");
    hexfloats(c.dir, 3);
    printf(", \"up\": ");
    hexfloats(c.up, 3);
    printf(", \"aov\": \"%a\", \"width\": %d, \"height\": %d}", (double)c.aov, c.width, c.height);
    printf(", \"lighting\": {\"n\": %d, \"lights\": ", L.n_lights);
    hexfloats(&L.lights[0][0], 3 * L.n_lights);
    printf(", \"types\": [");
    for (int k = 0; k < L.n_lights; k++) printf("%s%d", k ? ", " : "", L.types[k]);
    printf("], \"Ka\": \"%a\", \"Kd\": \"%a\", \"n_ao\": %d, \"ao_radius\": \"%a\", \"shadows\": %d}",
           (double)L.Ka, (double)L.Kd, L.n_ao, (double)L.ao_radius, L.shadows);
    printf(", \"epsilon\": \"%a\", \"volumes\": [", (double)r.vis->epsilon);
    for (size_t m = 0; m < r.vis->volumes.size(); m++) {
        const VolumeVis &v = r.vis->volumes[m];
        gxy_tf tf = v.local_commit();
        printf("%s{\"counts\": [%d, %d, %d], \"colors\": ", m ? ", " : "", v.volume->counts[0],
               v.volume->counts[1], v.volume->counts[2]);
        hexfloats(tf.colors, 3 * GXY_TF_SIZE);
        printf(", \"opacities\": ");
        hexfloats(tf.opacities, GXY_TF_SIZE);
        printf(", \"range\": ");
        hexfloats(tf.range, 2);
        printf(", \"slices\": %zu, \"isovalues\": %zu, \"volume_rendering\": %d}", v.slices.size(),
               v.isovalues.size(), v.volume_rendering ? 1 : 0);
    }
    printf("]}\n");
}

int main(int argc, char **argv) {
    int w = 0, h = 0, part[3] = {1, 1, 1}, device = 0, raylist_part = -1;
    bool describe_only = false;
    std::string prefix = "image", state;
    for (int k = 1; k < argc; k++) {
        std::string a = argv[k];
        if (a == "-s" && k + 2 < argc) {
            w = atoi(argv[++k]);
            h = atoi(argv[++k]);
        } else if (a == "-p" && k + 3 < argc) {
            for (int j = 0; j < 3; j++) part[j] = atoi(argv[++k]);
        } else if (a == "-o" && k + 1 < argc) {
            prefix = argv[++k];
        } else if (a == "-d" && k + 1 < argc) {
            device = atoi(argv[++k]);
        } else if (a == "-R" && k + 1 < argc) {
            raylist_part = atoi(argv[++k]);
        } else if (a == "-n") {
            describe_only = true;
        } else if (!a.empty() && a[0] != '-') {
            state = a;
        } else {
            return usage();
        }
    }
    if (state.empty()) return usage();
    try {
        RenderingSet set;
        set.renderings = LoadState(state, part, w, h);
        if (describe_only) {
            for (auto &r : set.renderings) describe(*r);
            fflush(stdout);
            return 0;
        }
        check(gxy_gpu_init(device, 0));
        set.Render();
        for (size_t k = 0; k < set.renderings.size(); k++) {
            Rendering &r = *set.renderings[k];
            char name[4096];
            snprintf(name, sizeof name, "%s_%05zu.rgba", prefix.c_str(), k);
            FILE *f = fopen(name, "wb");
            if (!f) throw std::runtime_error(std::string("cannot write ") + name);
            fwrite(r.framebuffer.data(), sizeof(float), r.framebuffer.size(), f);
            fclose(f);
            printf("{\"image\": \"%s\", \"width\": %d, \"height\": %d, \"primary\": %lld, \"shadow\": %lld, "
                   "\"ao\": %lld",
                   name, r.camera.width, r.camera.height, (long long)r.counters.primary_rays,
                   (long long)r.counters.shadow_rays, (long long)r.counters.ao_rays);
            if (raylist_part >= 0) {
                RayList rays = GenerateInitialRays(*r.vis, r.camera, raylist_part);
                gxy_lighting in = r.vis->lighting.c(), L;
                gxy_camera c = r.camera.c();
                check(gxy_resolve_lights(&in, &c, &L));
                Lighting resolved = r.vis->lighting;
                for (int j = 0; j < L.n_lights; j++) {
                    resolved.sources[j] = {L.lights[j][0], L.lights[j][1], L.lights[j][2]};
                    resolved.types[j] = L.types[j];
                }
                RayList sec = Trace(resolved, *r.vis, raylist_part, rays);
                long long hits = 0;
                for (int j = 0; j < rays.GetRayCount(); j++) hits += (rays.i[3][j] & GXY_RAY_SURFACE) ? 1 : 0;
                RayList again = sec;
                Trace(resolved, *r.vis, raylist_part, again);
                long long sec_hits = 0;
                for (int j = 0; j < again.GetRayCount(); j++) sec_hits += (again.i[3][j] & GXY_RAY_SURFACE) ? 1 : 0;
                printf(", \"raylist\": {\"partition\": %d, \"rays\": %d, \"hits\": %lld, \"secondary\": %d, "
                       "\"secondary_hits\": %lld}",
                       raylist_part, rays.GetRayCount(), hits, sec.GetRayCount(), sec_hits);
            }
            printf("}\n");
        }
        fflush(stdout);
        return 0;
    } catch (const GxyError &e) {
        fprintf(stderr, "gxywriter: library error %d: %s\n", e.code, e.what());
        return 1;
    } catch (const std::exception &e) {
        fprintf(stderr, "gxywriter: %s\n", e.what());
        return 1;
    }
}
