// Test-only: the binding a maintainer would add inside FCL (fcl::collide,
// fcl::continuousCollide and a broadphase manager forwarding to the C ABI), written
// against include/fclgpu.h with small stand-ins for the FCL types it touches.  The
// tests compile it (syntax and types only: no FCL, no GPU), so the documented calls
// keep matching the header's structs and signatures.
#include <cstdint>
#include <stdexcept>
#include <vector>

#include "fclgpu.h"

namespace standin {

// the parts of FCL's types the binding uses (math/, narrowphase/, broadphase/ headers)
struct Vector3d {
  double v[3];
  explicit Vector3d(const double* p) : v{p[0], p[1], p[2]} {}
};
struct Transform3d {
  double m[12];  // row-major 3x4
};
struct CollisionGeometry {};
template <class S>
struct Contact {
  Contact(const CollisionGeometry*, const CollisionGeometry*, int, int) {}
  Contact(const CollisionGeometry*, const CollisionGeometry*, int, int, const Vector3d&, const Vector3d&, S) {}
};
template <class S>
struct CollisionResult {
  std::vector<Contact<S>> contacts;
  void addContact(const Contact<S>& c) { contacts.push_back(c); }
  std::size_t numContacts() const { return contacts.size(); }
};
struct CollisionRequest {
  std::size_t num_max_contacts = 1;
  bool enable_statistics = false;
  bool enable_contact = false;
};
struct ContinuousCollisionRequest {
  std::size_t num_max_iterations = 10;
  double toc_err = 1e-4;
  int ccd_motion_type = FCLGPU_CCDM_TRANS;
  int ccd_solver_type = FCLGPU_CCDC_NAIVE;
};
struct ContinuousCollisionResult {
  bool is_collide = false;
  double time_of_contact = 1.0;
  Transform3d contact_tf1{}, contact_tf2{};
};
struct CollisionObject {
  const CollisionGeometry* geom;
  Transform3d tf;
  const CollisionGeometry* collisionGeometry() const { return geom; }
  const Transform3d& getTransform() const { return tf; }
};
struct DefaultCollisionData {
  CollisionRequest request;
  CollisionResult<double> result;
};

void to_3x4(const Transform3d& t, double* out) {
  for (int i = 0; i < 12; ++i) out[i] = t.m[i];
}
void append_3x4(std::vector<double>& v, const Transform3d& t) { v.insert(v.end(), t.m, t.m + 12); }
Transform3d from_3x4(const double* p) {
  Transform3d t;
  for (int i = 0; i < 12; ++i) t.m[i] = p[i];
  return t;
}

// inside fcl::collide for two BVHModel<OBBRSS<double>> (collision-inl.h:93-149)
void collide_meshes(const CollisionGeometry* model1, const CollisionGeometry* model2, fclgpu_mesh mirror1,
                    fclgpu_mesh mirror2, const CollisionObject* o1, const CollisionObject* o2,
                    const CollisionRequest& request, CollisionResult<double>& result) {
  fclgpu_mesh m[2] = {mirror1, mirror2};  // device mirrors cached per geometry + version
  int32_t pair[2] = {0, 1};
  double tf1[12], tf2[12];
  to_3x4(o1->getTransform(), tf1);
  to_3x4(o2->getTransform(), tf2);
  int32_t count;
  int64_t off[2];
  if (!request.enable_contact) {
    fclgpu_collide_request rq = {(int32_t)request.num_max_contacts, FCLGPU_FP32_RECHECK,
                                 request.enable_statistics, 0};
    std::vector<int32_t> pairs(2 * request.num_max_contacts);
    fclgpu_collide_result rs = {&count, off, pairs.data(), (int64_t)request.num_max_contacts, 0, 0, 0, 0};
    if (fclgpu_collide_batch(m, 2, pair, 1, 1, nullptr, tf1, tf2, &rq, &rs, nullptr) != FCLGPU_OK)
      throw std::runtime_error(fclgpu_last_error_detail());
    for (int i = 0; i < count; ++i)
      result.addContact(Contact<double>(model1, model2, pairs[2 * i], pairs[2 * i + 1]));
    return;
  }
  // enable_contact: contact geometry (mesh_collision_traversal_node-inl.h:579-600)
  const int64_t cap = (int64_t)request.num_max_contacts;
  std::vector<int32_t> ids(2 * cap);
  std::vector<double> pos(3 * cap), nrm(3 * cap), dep(cap);
  fclgpu_contact_result cr = {&count, off, ids.data(), pos.data(), nrm.data(), dep.data(), cap, 0};
  fclgpu_collide_request crq = {(int32_t)request.num_max_contacts, FCLGPU_FP32_RECHECK, 0, 0};
  if (fclgpu_collide_contacts(m, 2, pair, 1, 1, nullptr, tf1, tf2, &crq, &cr, nullptr) != FCLGPU_OK)
    throw std::runtime_error(fclgpu_last_error_detail());  // FCLGPU_ERR_CAPACITY: grow cap
  for (int i = 0; i < count; ++i)
    result.addContact(Contact<double>(model1, model2, ids[2 * i], ids[2 * i + 1], Vector3d(&pos[3 * i]),
                                      Vector3d(&nrm[3 * i]), dep[i]));
}

// fcl::continuousCollide on two meshes (continuous_collision-inl.h:436-469)
int continuous_collide_meshes(fclgpu_mesh mirror1, fclgpu_mesh mirror2, const Transform3d& tf1_beg,
                              const Transform3d& tf1_end, const Transform3d& tf2_beg, const Transform3d& tf2_end,
                              const ContinuousCollisionRequest& request, ContinuousCollisionResult& result) {
  fclgpu_mesh m[2] = {mirror1, mirror2};
  int32_t pair[2] = {0, 1};
  double a0[12], a1[12], b0[12], b1[12];
  to_3x4(tf1_beg, a0);
  to_3x4(tf1_end, a1);
  to_3x4(tf2_beg, b0);
  to_3x4(tf2_end, b1);
  fclgpu_ccd_request q = {(int64_t)request.num_max_iterations, request.toc_err, request.ccd_motion_type,
                          request.ccd_solver_type, FCLGPU_FP32_RECHECK, 0};
  int32_t hit;
  double toc, c1[12], c2[12];
  fclgpu_ccd_result r = {&hit, &toc, c1, c2, nullptr};
  const int rc = fclgpu_continuous_collide_batch(m, 2, pair, 1, 1, nullptr, a0, a1, b0, b1, &q, &r, nullptr);
  if (rc != FCLGPU_OK) return rc;  // FCLGPU_ERR_UNSUPPORTED: other solvers stay on FCL's CPU path
  result.is_collide = hit != 0;
  result.time_of_contact = toc;
  if (hit) {
    result.contact_tf1 = from_3x4(c1);
    result.contact_tf2 = from_3x4(c2);
  }
  return rc;
}

// a BroadPhaseCollisionManager forwarding registerObjects + setup, collide(query, data,
// DefaultCollisionFunction) and collide(data, DefaultCollisionFunction)
// (broadphase_collision_manager.h:65-122)
int manager_collide(fclgpu_shapeset shapeset, const std::vector<fclgpu_mesh>& mesh_handles,
                    const std::vector<CollisionObject*>& objs, fclgpu_geometry_ref (*ref_of)(const CollisionGeometry*),
                    const CollisionObject* query, DefaultCollisionData& data, DefaultCollisionData& self_data,
                    const CollisionGeometry* (*geom)(int32_t)) {
  std::vector<fclgpu_geometry_ref> refs;
  std::vector<double> tf;  // 12 doubles per object
  for (auto* o : objs) {
    refs.push_back(ref_of(o->collisionGeometry()));
    append_3x4(tf, o->getTransform());
  }
  fclgpu_broadphase bp;
  int rc = fclgpu_broadphase_create(shapeset, mesh_handles.data(), (int32_t)mesh_handles.size(), refs.data(),
                                    (int32_t)refs.size(), tf.data(), &bp);
  if (rc != FCLGPU_OK) return rc;
  // collide(query, &data, DefaultCollisionFunction)
  fclgpu_geometry_ref q = ref_of(query->collisionGeometry());
  double qtf[12];
  to_3x4(query->getTransform(), qtf);
  fclgpu_broadphase_collide_request rq = {(int64_t)data.request.num_max_contacts, FCLGPU_FP32_RECHECK, 0};
  int64_t n;
  int32_t nobj, first;
  fclgpu_broadphase_collide_result rs = {&n, &nobj, &first, 0, 0};
  rc = fclgpu_broadphase_collide(bp, &q, 1, qtf, &rq, &rs, nullptr);  // n == data.result.numContacts()
  // collide(cdata, DefaultCollisionFunction): every contacting pair once, grouped by the
  // higher index
  const int64_t n_objects = (int64_t)objs.size();
  int64_t cap = 1024;
  fclgpu_broadphase_contacts_request cq = {(int64_t)self_data.request.num_max_contacts, FCLGPU_FP32_RECHECK, 0};
  std::vector<int64_t> cnt(n_objects), off(n_objects + 1);
  std::vector<int32_t> trip(3 * cap);
  fclgpu_broadphase_contacts_result cr = {cnt.data(), off.data(), trip.data(), cap, 0, 0, 0};
  if (rc == FCLGPU_OK) rc = fclgpu_broadphase_self_collide_contacts(bp, &cq, &cr, nullptr);
  for (int64_t o2 = 0; rc == FCLGPU_OK && o2 < n_objects; ++o2)
    for (int64_t k = off[o2]; k < off[o2 + 1] && self_data.result.numContacts() < self_data.request.num_max_contacts;
         ++k)
      self_data.result.addContact(Contact<double>(geom(trip[3 * k]), geom((int32_t)o2), trip[3 * k + 1],
                                                  trip[3 * k + 2]));
  fclgpu_broadphase_destroy(bp);
  return rc;
}

}  // namespace standin
