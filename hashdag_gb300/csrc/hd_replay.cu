// Replays: the reference's recorded edit and camera streams.
//
// ReplayManager (replay.h:462-635) reads a CSV of actions, one per line,
// "<Type>,<cell>,<cell>..." (no quoting; trailing empty cells dropped), and
// replays them frame by frame: every action up to and including the next
// EndFrame.  The actions (replay.h:12-460) and their effect (replay.cpp:
// 5-100): the camera's location and rotation, the tool parameters, the
// sphere / cube / copy / fill / paint edits and undo / redo.  Positions and
// radii were recorded on a scene of REPLAY_DEPTH levels and are scaled by
// float(1 << depth) / float(1 << REPLAY_DEPTH) on replay.  A frame's camera
// is get_trace_params (dag_tracer.cu:71-113) of the view at its EndFrame.
#include <cmath>
#include <cstdio>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "hd_ctx.h"

struct hd_replay {
    struct Action {
        uint32_t type;
        std::vector<float> f;     // the float cells, in order
        std::vector<uint32_t> i;  // the integer cells, in order ((uint32)std::stoi)
        bool flag = false;        // add / enableSwirl
    };
    std::vector<Action> actions;
    uint64_t frames = 0;
    uint64_t next = 0;
    // the engine state the actions set (Engine::view, Engine::config)
    double position[3] = {0, 0, 0};
    double rotation[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    uint32_t tool_path[3] = {0, 0, 0}, tool_source[3] = {0, 0, 0}, tool_dest[3] = {0, 0, 0};
    float tool_radius = 0;
    uint32_t tool = 0;
};

namespace hd {
namespace {

const char* const kNames[] = {"SetLocation", "SetRotation", "SetToolParameters", "EditSphere", "EditCube", "EditCopy",
                              "EditFill",    "EditPaint",   "Undo",              "Redo",       "EndFrame"};

int type_of(const std::string& s)
{
    for (int k = 0; k <= HD_REPLAY_END_FRAME; k++)
        if (s == kNames[k])
            return k;
    return -1;
}

bool is_bool(const std::string& s) { return s == "true" || s == "false" || s == "TRUE" || s == "FALSE"; }
bool bool_of(const std::string& s) { return s == "true" || s == "TRUE"; }

// IReplayAction::load of each action (replay.h:112-460): cell counts, stof /
// stoi conversions.
hd_replay::Action parse(uint32_t type, const std::vector<std::string>& d, uint64_t line)
{
    auto fail = [&](const char* why) {
        return StatusError{HD_ERR_INVALID, "replay line " + std::to_string(line) + " (" + kNames[type] + "): " + why};
    };
    auto need = [&](size_t n) {
        if (d.size() != n)
            throw fail(("expects " + std::to_string(n) + " cells").c_str());
    };
    hd_replay::Action a;
    a.type = type;
    try {
        switch (type) {
        case HD_REPLAY_SET_LOCATION:
            need(3);
            for (int k = 0; k < 3; k++)
                a.f.push_back(std::stof(d[k]));
            break;
        case HD_REPLAY_SET_ROTATION:
            need(9);
            for (int k = 0; k < 9; k++)
                a.f.push_back(std::stof(d[k]));
            break;
        case HD_REPLAY_SET_TOOL_PARAMETERS:
            need(11);
            for (int k = 0; k < 9; k++)
                a.i.push_back(uint32_t(std::stoi(d[k])));
            a.f.push_back(std::stof(d[9]));
            a.i.push_back(uint32_t(std::stoi(d[10])));
            break;
        case HD_REPLAY_EDIT_SPHERE:
        case HD_REPLAY_EDIT_CUBE:
            need(5);
            for (int k = 0; k < 4; k++)
                a.f.push_back(std::stof(d[k]));
            if (!is_bool(d[4]))
                throw fail("the last cell is not a boolean");
            a.flag = bool_of(d[4]);
            break;
        case HD_REPLAY_EDIT_COPY:
            if (d.size() != 10 && d.size() != 21)
                throw fail("expects 10 or 21 cells");
            for (int k = 0; k < 10; k++)
                a.f.push_back(std::stof(d[k]));
            if (d.size() == 21) {
                for (int k = 10; k < 19; k++)
                    a.f.push_back(std::stof(d[k]));
                if (!is_bool(d[19]))
                    throw fail("cell 20 is not a boolean");
                a.flag = bool_of(d[19]);
                a.f.push_back(std::stof(d[20]));
            }
            break;
        case HD_REPLAY_EDIT_FILL:
        case HD_REPLAY_EDIT_PAINT:
            need(4);
            for (int k = 0; k < 4; k++)
                a.f.push_back(std::stof(d[k]));
            break;
        default: // Undo, Redo, EndFrame: cells are ignored
            break;
        }
    } catch (const std::logic_error&) {
        throw fail("a cell is not a number");
    }
    return a;
}

// ReplayManager::load_csv (replay.h:526-567)
void load(hd_replay& r, std::istream& is)
{
    std::vector<std::string> data;
    uint64_t line = 0;
    char c;
    while (is.get(c)) {
        if (c == '\n') {
            line++;
            if (data.empty())
                throw StatusError{HD_ERR_INVALID, "replay line " + std::to_string(line) + " is empty"};
            const int type = type_of(data[0]);
            if (type < 0)
                throw StatusError{HD_ERR_INVALID,
                                  "replay line " + std::to_string(line) + ": unknown action " + data[0]};
            data.erase(data.begin());
            if (type == HD_REPLAY_END_FRAME)
                r.frames++;
            while (!data.empty() && data.back().empty())
                data.pop_back();
            r.actions.push_back(parse(uint32_t(type), data, line));
            data.clear();
        } else if (c == ',') {
            data.emplace_back();
        } else {
            if (data.empty())
                data.emplace_back();
            data.back().push_back(c);
        }
    }
}

// std::to_string of a float / int (IReplayAction::write, replay.h:112-460)
std::string str(float v) { return std::to_string(v); }
std::string str(uint32_t v) { return std::to_string(v); }

// ReplayManager::write_csv (replay.h:504-520)
void write(const hd_replay& r, std::ostream& os)
{
    for (const auto& a : r.actions) {
        os << kNames[a.type];
        std::vector<std::string> d;
        switch (a.type) {
        case HD_REPLAY_SET_LOCATION:
        case HD_REPLAY_SET_ROTATION:
        case HD_REPLAY_EDIT_FILL:
        case HD_REPLAY_EDIT_PAINT:
            for (float v : a.f)
                d.push_back(str(v));
            break;
        case HD_REPLAY_SET_TOOL_PARAMETERS:
            for (int k = 0; k < 9; k++)
                d.push_back(str(a.i[k]));
            d.push_back(str(a.f[0]));
            d.push_back(str(a.i[9]));
            break;
        case HD_REPLAY_EDIT_SPHERE:
        case HD_REPLAY_EDIT_CUBE:
            for (float v : a.f)
                d.push_back(str(v));
            d.push_back(a.flag ? "true" : "false");
            break;
        case HD_REPLAY_EDIT_COPY: {
            // the writer always emits the transform (identity when the line
            // had none), the swirl flag and its period (default 1)
            for (int k = 0; k < 10; k++)
                d.push_back(str(a.f[k]));
            const float identity[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
            for (int k = 0; k < 9; k++)
                d.push_back(str(a.f.size() == 20 ? a.f[10 + k] : identity[k]));
            d.push_back(a.flag ? "true" : "false");
            d.push_back(str(a.f.size() == 20 ? a.f[19] : 1.0f));
            break;
        }
        default:
            break;
        }
        for (auto& s : d)
            os << "," << s;
        os << "\n";
    }
}

// get_trace_params (dag_tracer.cu:71-113): the camera frame (right = -row
// 0, up = row 1, forward = row 2 of the rotation, camera_view.h:13-27) at
// fov_degrees, mapped into the voxel space of a 2^levels scene whose
// bounding box is info.
hd_camera camera_from_view(const double position[3], const double rotation[9], double fov_degrees, uint32_t levels,
                           const hd_dag_info& info, uint32_t width, uint32_t height)
{
    const double* p = position;
    const double* m = rotation;
    const double right[3] = {-m[0], -m[1], -m[2]}, up[3] = {m[3], m[4], m[5]}, fwd[3] = {m[6], m[7], m[8]};
    const double fov = fov_degrees / 2.0 * (double(M_PI) / 180.);
    const double aspect = double(width) / double(height);
    hd_camera cam{};
    double bl[3], br[3], tl[3];
    for (int a = 0; a < 3; a++) {
        const double X = right[a] * sin(fov) * aspect, Y = up[a] * sin(fov), Z = fwd[a] * cos(fov);
        bl[a] = p[a] + Z - Y - X;
        br[a] = p[a] + Z - Y + X;
        tl[a] = p[a] + Z + Y - X;
    }
    for (int a = 0; a < 3; a++) {
        const double translation = -info.aabb_min[a];
        const double scale = double(1u << levels) / (info.aabb_max[a] - info.aabb_min[a]);
        const double fp = (p[a] + translation) * scale, fbl = (bl[a] + translation) * scale,
                     ftl = (tl[a] + translation) * scale, fbr = (br[a] + translation) * scale;
        cam.position[a] = fp;
        cam.ray_min[a] = fbl;
        cam.ray_ddx[a] = (fbr - fbl) * (1.0 / width);
        cam.ray_ddy[a] = (ftl - fbl) * (1.0 / height);
    }
    return cam;
}

// the replay's view, with CameraView::fov (60 degrees, camera_view.h:9)
hd_camera camera_of(const hd_replay& r, uint32_t levels, const hd_replay_config& cfg)
{
    return camera_from_view(r.position, r.rotation, double(60.f), levels, cfg.info, cfg.width, cfg.height);
}

// IReplayAction::apply (replay.cpp:5-100) on the context
void apply(hd_ctx* c, hd_replay& r, const hd_replay::Action& a, float scale, uint32_t* edits)
{
    auto scaled = [&](int k) { return a.f[k] * scale; };
    hd_edit e{};
    switch (a.type) {
    case HD_REPLAY_SET_LOCATION:
        for (int k = 0; k < 3; k++)
            r.position[k] = a.f[k];
        return;
    case HD_REPLAY_SET_ROTATION:
        for (int k = 0; k < 9; k++)
            r.rotation[k] = a.f[k];
        return;
    case HD_REPLAY_SET_TOOL_PARAMETERS:
        for (int k = 0; k < 3; k++) {
            r.tool_path[k] = uint32_t(float(a.i[k]) * scale);
            r.tool_source[k] = uint32_t(float(a.i[3 + k]) * scale);
            r.tool_dest[k] = uint32_t(float(a.i[6 + k]) * scale);
        }
        r.tool_radius = a.f[0] * scale;
        r.tool = a.i[9];
        return;
    case HD_REPLAY_EDIT_SPHERE:
    case HD_REPLAY_EDIT_CUBE:
        e.tool = a.type == HD_REPLAY_EDIT_SPHERE ? (a.flag ? HD_TOOL_SPHERE_ADD : HD_TOOL_SPHERE_REMOVE)
                                                 : (a.flag ? HD_TOOL_BOX_ADD : HD_TOOL_BOX_REMOVE);
        e.center[0] = scaled(0);
        e.center[1] = scaled(1);
        e.center[2] = scaled(2);
        e.radius = scaled(3);
        break;
    case HD_REPLAY_EDIT_COPY:
        // CopyEditorWithDecompression ignores the transform and the swirl
        e.tool = HD_TOOL_COPY;
        for (int k = 0; k < 3; k++) {
            e.center[k] = scaled(k);
            e.source[k] = scaled(3 + k);
            e.dest[k] = scaled(6 + k);
        }
        e.radius = scaled(9);
        break;
    case HD_REPLAY_EDIT_FILL:
        e.tool = HD_TOOL_FILL;
        e.center[0] = scaled(0);
        e.center[1] = scaled(1);
        e.center[2] = scaled(2);
        e.radius = scaled(3);
        break;
    case HD_REPLAY_EDIT_PAINT:
        e.tool = HD_TOOL_SPHERE_PAINT;
        e.rgb = 0xFF0000u; // SpherePaintEditor's blue (hash_dag_editors.h:327)
        e.center[0] = scaled(0);
        e.center[1] = scaled(1);
        e.center[2] = scaled(2);
        e.radius = scaled(3);
        break;
    case HD_REPLAY_UNDO: // HashDAGUndoRedo::undo / redo: nothing to undo is no error
        undo_step(c, false);
        return;
    case HD_REPLAY_REDO:
        undo_step(c, true);
        return;
    default:
        return;
    }
    edit_one(c, e, nullptr);
    if (edits)
        (*edits)++;
}

} // namespace
} // namespace hd

using namespace hd;

extern "C" {

hd_status hd_camera_from_view(const double position[3], const double rotation[9], double fov_degrees, uint32_t levels,
                              const hd_dag_info* info, uint32_t width, uint32_t height, hd_camera* out)
{
    if (!position || !rotation || !info || !out || !width || !height || levels > 31 || !(fov_degrees > 0.0) ||
        !(fov_degrees < 180.0))
        return HD_ERR_INVALID;
    for (int a = 0; a < 3; a++)
        if (!(info->aabb_max[a] > info->aabb_min[a]))
            return HD_ERR_INVALID;
    *out = camera_from_view(position, rotation, fov_degrees, levels, *info, width, height);
    return HD_OK;
}

hd_status hd_replay_load(const char* path, hd_replay** out)
{
    if (!path || !out)
        return HD_ERR_INVALID;
    *out = nullptr;
    std::ifstream is(path, std::ios::binary);
    if (!is.is_open())
        return HD_ERR_IO;
    hd_replay* r = new (std::nothrow) hd_replay();
    if (!r)
        return HD_ERR_OOM;
    const hd_status st = guarded(nullptr, [&] { load(*r, is); });
    if (st != HD_OK) {
        delete r;
        return st;
    }
    *out = r;
    return HD_OK;
}

hd_status hd_replay_load_text(const char* text, uint64_t n, hd_replay** out)
{
    if (!text || !out)
        return HD_ERR_INVALID;
    *out = nullptr;
    std::istringstream is(std::string(text, n));
    hd_replay* r = new (std::nothrow) hd_replay();
    if (!r)
        return HD_ERR_OOM;
    const hd_status st = guarded(nullptr, [&] { load(*r, is); });
    if (st != HD_OK) {
        delete r;
        return st;
    }
    *out = r;
    return HD_OK;
}

hd_status hd_replay_free(hd_replay* r)
{
    delete r;
    return HD_OK;
}

hd_status hd_replay_info(const hd_replay* r, uint64_t* n_actions, uint64_t* n_frames, uint64_t* next_action)
{
    if (!r)
        return HD_ERR_INVALID;
    if (n_actions)
        *n_actions = r->actions.size();
    if (n_frames)
        *n_frames = r->frames;
    if (next_action)
        *next_action = r->next;
    return HD_OK;
}

hd_status hd_replay_get_action(const hd_replay* r, uint64_t index, hd_replay_action* out)
{
    if (!r || !out || index >= r->actions.size())
        return HD_ERR_INVALID;
    const auto& a = r->actions[index];
    *out = hd_replay_action{};
    out->type = a.type;
    out->flag = a.flag ? 1u : 0u;
    out->n_floats = uint32_t(a.f.size());
    out->n_ints = uint32_t(a.i.size());
    for (size_t k = 0; k < a.f.size() && k < 20; k++)
        out->floats[k] = a.f[k];
    for (size_t k = 0; k < a.i.size() && k < 10; k++)
        out->ints[k] = a.i[k];
    return HD_OK;
}

hd_status hd_replay_write(const hd_replay* r, const char* path)
{
    if (!r || !path)
        return HD_ERR_INVALID;
    std::ofstream os(path, std::ios::binary);
    if (!os.is_open())
        return HD_ERR_IO;
    write(*r, os);
    os.close();
    return os.good() ? HD_OK : HD_ERR_IO;
}

hd_status hd_replay_reset(hd_replay* r)
{
    if (!r)
        return HD_ERR_INVALID;
    r->next = 0;
    return HD_OK;
}

hd_status hd_replay_frame(hd_ctx* c, hd_replay* r, const hd_replay_config* cfg, hd_camera* cam, uint32_t* edits)
{
    if (!c || !r || !cfg || !cfg->width || !cfg->height || cfg->replay_depth > 31)
        return HD_ERR_INVALID;
    if (r->next >= r->actions.size())
        return HD_ERR_STATE;
    if (edits)
        *edits = 0;
    return guarded(c, [&] {
        const float scale = float(1u << c->cfg.depth) / float(1u << cfg->replay_depth);
        // ReplayManager::replay_frame (replay.h:479-495): up to and including
        // the next EndFrame
        uint32_t type;
        do {
            const auto& a = r->actions[r->next];
            type = a.type;
            apply(c, *r, a, scale, edits);
            r->next++;
        } while (type != HD_REPLAY_END_FRAME && r->next < r->actions.size());
        if (cam)
            *cam = camera_of(*r, c->cfg.depth, *cfg);
    });
}

} // extern "C"
