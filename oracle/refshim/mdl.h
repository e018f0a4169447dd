// Test infrastructure: the declarations of pkdgrav3's MDL runtime that the reference's
// services and src/services/pst.h name, so the reference's CPU services compile unchanged
// without MDL. Nothing here sends a message: the test driver calls each rank's Service()
// itself and sums the ranks' outputs with the services' own Combine(), which is what MDL's
// request/reply traversal does (src/services/TraversePST.cpp:37-44).
#ifndef ORB_REFSHIM_MDL_H
#define ORB_REFSHIM_MDL_H

#include <cstdint>

typedef void *MDL;

inline int mdlSelf(MDL) { return 0; }
inline int mdlCores(MDL) { return 1; }

namespace mdl {

class mdlClass {};

class BasicService {
   public:
    BasicService(int service_id, int nInBytes, int nOutBytes, const char *service_name = "")
        : id_(service_id), n_in_(nInBytes), n_out_(nOutBytes), name_(service_name) {}
    virtual ~BasicService() = default;
    int getServiceID() const { return id_; }
    int getMaxBytesIn() const { return n_in_; }
    int getMaxBytesOut() const { return n_out_; }
    const char *getServiceName() const { return name_; }

   protected:
    virtual int operator()(int nIn, void *pIn, void *pOut) = 0;

   private:
    int id_, n_in_, n_out_;
    const char *name_;
};

}  // namespace mdl

#endif
